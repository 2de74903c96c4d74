"""Run the pyBELLA reference's rising bubble to t_end and record its state
(fixture generation only; the fixture is committed, the reference is not
needed at test time).

    python tests/golden/make_fullrun.py /path/to/pyBELLA [--stop TOUT] [--resume]
    python tests/golden/make_fullrun.py --oracle


The case is the reference's ``inputs/rising_bubble.py`` (160x80 cells, CFL 0.5,
'CFLfixed', output times 0.1 ... 1.0 every 0.01 in units of t_ref = 1000 s),
pseudo-incompressible with the projection's BiCGStab at tol 1e-10, exactly
as ``make_golden.py`` sets it up.  The output loop is the reference driver's
for one member (``src/__main__.py:198-393``): ``time_update.do`` once per
output time, the step counter carried across calls (``mem[3][0] = mem[3][1]``,
``:229-230``) and ``t`` set to the output time rounded to three decimals
(``:266, 388``).

The reference runs here through ``refshim`` with numba stubbed, i.e. as plain
Python: about 45 s per solve, a few hours for the whole run.  The state is
written after every tenth output time (``fullrun_kat.npz``: theta = rhoY / rho
at t = 0.1, 0.2, ..., all fields and p2 at the last output time reached, the
step count and t), so an interrupted run still leaves a usable fixture.
``--resume`` continues such a run from the last state written: a time step of
the reference depends on nothing but ``Sol``, ``mpv.p2_nodes``, ``t`` and the
step count (everything else it reads is the static background or is recomputed
at the step's start), so the continuation is the same run.

``--oracle`` runs the same case through the oracle's restatement of the step and
its output loop (``oracle/step2d.py``: ``run_outputs``, pinned to the reference's
``do``) in a few minutes and writes ``fullrun_oracle_kat.npz`` with the same
keys, from the same initial state (the reference's, when ``fullrun_kat.npz``
exists).  scipy's BiCGStab takes its inner products from BLAS, whose summation
order depends on the thread count, so the two runs agree to rounding, not bit
for bit, unless both use the same count; the committed oracle fixture was made
with OPENBLAS_NUM_THREADS=1, the reference's with the host's default (8).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refshim  # noqa: E402

FIELDS = ["rho", "rhou", "rhov", "rhow", "rhoY", "rhoX"]


def oracle_main():
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import cases, step2d
    grid, prm, Sol, p2, hn, hc, sf = cases.rising_bubble()
    S0c = np.broadcast_to(hc["S0"][None, :], grid.elem_sc).copy()
    ref = os.path.join(HERE, "fullrun_kat.npz")
    if os.path.exists(ref):                        # the reference's initial state and backgrounds
        d = np.load(ref)
        Sol = {k: d["in_" + k].copy() for k in FIELDS}
        p2 = d["p2_in"].copy()
        hn, hc, S0c = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"]), d["S0c"]
    rec = {"in_" + k: np.copy(Sol[k]) for k in FIELDS}
    rec.update(p2_in=np.copy(p2), S0n=np.copy(hn["S0"]), rhoY0=np.copy(hc["rhoY0"]), S0c=np.copy(S0c),
               meta=np.array([grid.inx, grid.iny, prm.Msq, prm.g, prm.gamm, 1000.0, prm.tol, 0.5]))
    touts = np.arange(0.0, 1.01, 0.01)[10:]                      # inputs/rising_bubble.py:25
    thetas, ts = [], []
    t0 = time.time()

    def on_output(t, S, p, step):
        if int(round(t * 100)) % 10 == 0:
            thetas.append(S["rhoY"] / S["rho"])
            ts.append(t)
            print("tout %.3f  step %d  %.0f s" % (t, step, time.time() - t0), flush=True)
    Sol, t, step = step2d.run_outputs(Sol, p2, touts, 10000, grid, prm, hn, hc, S0c, sf, 1000.0,
                                      on_output=on_output)
    rec["theta"], rec["theta_t"] = np.array(thetas), np.array(ts)
    for k in FIELDS:
        rec["out_" + k] = np.copy(Sol[k])
    rec.update(out_p2=np.copy(p2), out_t=np.array(t), out_step=np.array(step))
    np.savez_compressed(os.path.join(HERE, "fullrun_oracle_kat.npz"), **rec)


def main():
    if "--oracle" in sys.argv:
        return oracle_main()
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if not args:
        raise SystemExit("usage: make_fullrun.py REFERENCE_ROOT [--stop TOUT] [--resume]")
    stop = None
    if "--stop" in sys.argv:
        stop = float(sys.argv[sys.argv.index("--stop") + 1])
        args = [a for a in args if a != sys.argv[sys.argv.index("--stop") + 1]]
    refshim.install(args[0])
    sys.path.insert(0, os.path.dirname(HERE))
    from make_golden import _rb_setup_sized
    import dycore.discretisation.time_update as dis_time_update
    import dycore.utils.variable as var
    from data_assimilation import blending as da_blending

    ud, elem, node, Sol, th, mpv = _rb_setup_sized(161, 81)
    flux = np.empty((3), dtype=object)
    flux[0] = var.States(elem.sfx, ud)
    flux[1] = var.States(elem.sfy, ud)
    bld = da_blending.Blend(ud)
    rec = {"in_" + k: np.copy(getattr(Sol, k)) for k in FIELDS}
    rec["p2_in"] = np.copy(mpv.p2_nodes)
    rec["S0n"] = np.copy(mpv.HydroState_n.S0)
    rec["rhoY0"] = np.copy(mpv.HydroState.rhoY0)
    rec["S0c"] = np.copy(mpv.HydroState.get_S0c(elem))
    rec["meta"] = np.array([161, 81, ud.Msq, ud.gravity_strength[1], th.gamm, ud.t_ref, ud.tol, ud.CFL])
    out = os.path.join(HERE, "fullrun_kat.npz")
    steps = [0, 0]
    t, t0 = 0.0, time.time()
    thetas, touts_rec = [], []
    if "--resume" in sys.argv and os.path.exists(out):
        d = np.load(out)
        for k in FIELDS:                      # the run started from this very state
            assert np.array_equal(d["in_" + k], rec["in_" + k]), k
        for k in FIELDS:
            getattr(Sol, k)[...] = d["out_" + k]
        mpv.p2_nodes[...] = d["out_p2"]
        t = float(d["out_t"])
        steps = [int(d["out_step"]), int(d["out_step"])]
        thetas, touts_rec = list(d["theta"]), [float(v) for v in d["theta_t"]]
        print("resumed at t = %.3f, step %d" % (t, steps[1]), flush=True)
    for n, tout in enumerate(ud.tout):
        if float(np.around(tout, 3)) <= t:
            continue
        steps[0] = steps[1]                                         # __main__.py:229-230
        ret = dis_time_update.do(Sol, flux, mpv, t, tout, ud, elem, node, steps, th, bld, None, False)
        Sol, flux, mpv, steps = ret[0], ret[1], ret[2], list(ret[3])
        t = float(np.around(tout, 3))                              # __main__.py:266, 388
        print("tout %.3f  step %d  %.0f s" % (t, steps[1], time.time() - t0), flush=True)
        if n % 10 == 0 or n == len(ud.tout) - 1 or (stop is not None and t >= stop):
            thetas.append(Sol.rhoY / Sol.rho)
            touts_rec.append(t)
            rec["theta"] = np.array(thetas)
            rec["theta_t"] = np.array(touts_rec)
            for k in FIELDS:
                rec["out_" + k] = np.copy(getattr(Sol, k))
            rec["out_p2"] = np.copy(mpv.p2_nodes)
            rec["out_t"] = np.array(t)
            rec["out_step"] = np.array(steps[1])
            np.savez_compressed(out, **rec)
            print("  written at t = %.3f" % t, flush=True)
        if stop is not None and t >= stop:
            break


if __name__ == "__main__":
    main()
