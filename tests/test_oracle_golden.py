"""Pin the CPU oracle against the reference's own outputs (committed fixtures).

The fixtures were produced by importing the pyBELLA reference
(tests/golden/make_golden.py).  The oracle restates the reference's FP64
arithmetic in the same operation order, so most comparisons are exact.
"""
import numpy as np
import pytest

from conftest import golden, lap3d_case, step2d_case
from oracle import cases, nodal2d as n2, nodal3d as n3
from oracle.krylov import bicgstab_legacy, true_relres

FIELDS = ["rho", "rhou", "rhov", "rhow", "rhoY", "rhoX"]


def test_lap2d_matches_reference_kat():
    d = np.load(golden("lap2d_kat.npz"))
    for c in range(3):
        g = lambda k: d["c%d_%s" % (c, k)]
        nx, ny, xw, yw, dx, dy = g("meta")
        op = dict(hplusx=g("hx"), hplusy=g("hy"), hcenter=g("hc"),
                  cor=(g("cxx"), g("cyy"), g("cxy"), g("cyx")), diag_inv=g("dinv"),
                  nx=int(nx), ny=int(ny), dx=dx, dy=dy, x_wall=bool(xw), y_wall=bool(yw))
        y = n2.lap2d_gather(g("p"), op)
        np.testing.assert_array_equal(y, g("y"))


def test_precon_diag_matches_reference_kat():
    d = np.load(golden("diag_kat.npz"))
    dx, dy = d["meta"]
    out = n2.precon_diag_prepare(d["wplus"], d["wcenter"], dx, dy)
    np.testing.assert_array_equal(out, d["diag_inv"])


@pytest.mark.parametrize("tag", ["a", "b", "c", "d"])
def test_lap3d_matches_reference_kat(tag):
    """The reference's lap3D on random operands (periodic/wall mixes, Coriolis
    cross terms): the oracle reproduces the inner nodes bit for bit and the
    reference's outer node shell is zero."""
    d = np.load(golden("lap3d_kat.npz"))
    op, p, y = lap3d_case(d, tag)
    np.testing.assert_array_equal(n3.lap3d(p, op).reshape(y[1:-1, 1:-1, 1:-1].shape), y[1:-1, 1:-1, 1:-1])
    shell = y.copy()
    shell[1:-1, 1:-1, 1:-1] = 0.0
    assert not shell.any()


def test_lap3d_reference_overwrites_the_periodic_seam():
    """Case d has unequal seam values: lap3D replaces inner node 0 by inner node
    n-1 along each periodic axis before differencing, so its output is the
    operator applied to the seam-copied vector, not to the vector given."""
    d = np.load(golden("lap3d_kat.npz"))
    op, p_raw, y = lap3d_case(d, "d", seam_copy=False)
    _, p_seam, _ = lap3d_case(d, "d")
    inner = y[1:-1, 1:-1, 1:-1].reshape(-1)
    assert not np.array_equal(p_raw, p_seam)
    np.testing.assert_array_equal(n3.lap3d(p_seam, op), inner)
    assert not np.allclose(n3.lap3d(p_raw, op), inner)


def test_precon_diag_3d_matches_reference_kat():
    d = np.load(golden("diag3d_kat.npz"))
    dx, dy, dz = d["meta"]
    w = d["wplus"]
    out = n3.precon_diag_3d(w[0], w[1], w[2], d["wcenter"], dx, dy, dz)
    np.testing.assert_allclose(out, d["diag_inv"], rtol=1e-14, atol=0)


@pytest.mark.parametrize("tag", ["ww", "pw", "wp", "pwp", "www", "wwp", "pww"])
def test_scale_wall_node_values_matches_reference_kat(tag):
    """Wall/periodic mixes in 2D and 3D, factors 0.5 and 2: with two wall axes the
    reference's index carries over, and the oracle reproduces that."""
    import types
    d = np.load(golden("wall_kat.npz"))
    a = d[tag + "_in"]
    grid = types.SimpleNamespace(igs=[2] * a.ndim,
                                 bdry=[n2.WALL if w else n2.PERIODIC for w in d[tag + "_walls"]])
    for f, name in ((0.5, "half"), (2.0, "two")):
        b = a.copy()
        n2.scale_wall_node_values(b, grid, f)
        np.testing.assert_array_equal(b, d["%s_%s" % (tag, name)])


@pytest.mark.parametrize("tag", ["a", "b"])
def test_projection_pieces_3d_match_reference_kat(tag):
    """The 3D projection pieces (boundary data, coefficients, divergence with its
    x-sign, ghost nodes, correction with Coriolis, the explicit part with
    background wind) reproduce the reference's outputs bit for bit on
    periodic/wall and wall/wall states."""
    from conftest import proj3d_case
    from oracle import proj3d as o3
    d = np.load(golden("proj3d_kat.npz"))
    grid, prm, dt, S0n, hc, sf = proj3d_case(d, tag)
    Sol = {k: d["%s_in_%s" % (tag, k)].copy() for k in FIELDS}
    o3.set_explicit_boundary_data(Sol, grid, prm, hc, sf)
    for k in FIELDS:
        np.testing.assert_array_equal(Sol[k], d["%s_bd_%s" % (tag, k)], err_msg="boundary " + k)
    S = {k: v.copy() for k, v in Sol.items()}
    wplus, wcenter, _ = o3.operator_coefficients_nodes(S, S0n, grid, prm, dt)
    np.testing.assert_array_equal(wplus, d[tag + "_wplus"])
    np.testing.assert_array_equal(wcenter, d[tag + "_wcenter"])
    np.testing.assert_array_equal(o3.divergence_nodes(S, grid), d[tag + "_div"])
    for k in ("rhou", "rhov", "rhow"):
        np.testing.assert_array_equal(S[k], d["%s_dv_%s" % (tag, k)])
    q = d[tag + "_p"].copy()
    o3.set_ghostnodes_p2(q, grid)
    np.testing.assert_array_equal(q, d[tag + "_gn"])
    S = {k: v.copy() for k, v in Sol.items()}
    o3.correction_nodes(S, q, S0n, grid, prm, dt, 1)
    for k in FIELDS:
        np.testing.assert_array_equal(S[k], d["%s_cr_%s" % (tag, k)], err_msg="correction " + k)
    S = {k: v.copy() for k, v in Sol.items()}
    o3.euler_backward_non_advective_expl_part(S, S0n, grid, prm, dt, hc, sf, wind=d[tag + "_wind"])
    for k in FIELDS:
        np.testing.assert_array_equal(S[k], d["%s_xp_%s" % (tag, k)], err_msg="explicit part " + k)


def _small_rb_state():
    d = np.load(golden("pieces_kat.npz"))
    inx, iny, dt = d["meta"]
    grid, prm, Sol, p2, hn, hc, sf = cases.rising_bubble(inx=int(inx), iny=int(iny))
    return d, grid, prm, hn, hc, sf, dt


def test_projection_pieces_match_reference_kat():
    d, grid, prm, hn, hc, sf, dt = _small_rb_state()
    Sol = {k: d["in_" + k].copy() for k in FIELDS}
    n2.set_explicit_boundary_data(Sol, grid, prm, hc, sf)
    for k in FIELDS:
        np.testing.assert_array_equal(Sol[k], d["bd_" + k], err_msg="boundary " + k)
    div = n2.divergence_nodes(Sol, grid)
    np.testing.assert_array_equal(div, d["div"])
    for k in FIELDS:
        np.testing.assert_array_equal(Sol[k], d["dv_" + k], err_msg="divergence side effect " + k)
    n2.correction_nodes(Sol, d["p"], hn["S0"], grid, prm, dt, 1)
    for k in FIELDS:
        np.testing.assert_allclose(Sol[k], d["cr_" + k], rtol=0, atol=1e-15, err_msg="correction " + k)
    q = d["p"].copy()
    n2.set_ghostnodes_p2(q, grid)
    np.testing.assert_array_equal(q, d["gn_pw"])
    g2 = n2.Grid2D(grid.inx, grid.iny, -1.0, 1.0, 0.0, 1.0, (n2.WALL, n2.PERIODIC))
    q2 = d["p"].copy()
    n2.set_ghostnodes_p2(q2, g2)
    np.testing.assert_array_equal(q2, d["gn_wp"])


def test_rising_bubble_background_matches_reference():
    d = np.load(golden("rising_bubble_step0.npz"))
    grid, prm, Sol, p2, hn, hc, sf = cases.rising_bubble()
    np.testing.assert_array_equal(hn["S0"], d["hydro_n_S0"])
    np.testing.assert_array_equal(hc["rhoY0"], d["hydro_c_rhoY0"])
    Msq, g, gamm = d["scalars"]
    assert prm.Msq == Msq and prm.g == g and prm.gamm == gamm


@pytest.mark.parametrize("tag", ["full", "half"])
def test_impl_part_matches_reference_rising_bubble(tag):
    d = np.load(golden("rising_bubble_step0.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble()
    Sol = {k: d["%s_in_%s" % (tag, k)].copy() for k in FIELDS}
    Sol0 = None
    if ("%s_sol0_rho" % tag) in d:
        Sol0 = {k: d["%s_sol0_%s" % (tag, k)].copy() for k in FIELDS}
    p2 = d[tag + "_p2_in"].copy()
    out = n2.impl_part(Sol, p2, hn["S0"], hc, sf, grid, prm, float(d[tag + "_dt"]), Sol0=Sol0)
    assert out["niter"] == int(d[tag + "_niter"])
    np.testing.assert_array_equal(out["rhs"], d[tag + "_rhs"])
    np.testing.assert_array_equal(p2, d[tag + "_p2_out"])
    for k in FIELDS:
        np.testing.assert_array_equal(Sol[k], d["%s_out_%s" % (tag, k)], err_msg=k)
    assert true_relres(out["op"], out["x"], out["rhs_inner"]) <= prm.tol


@pytest.mark.parametrize("tag", ["ww", "cor"])
def test_impl_part_matches_reference_walls_and_coriolis(tag):
    """The whole 2D step with walls in x and y (the wall-scaling index carry-over,
    x-wall ghost cells and nodes) and with Coriolis cross terms in the
    compressible regime: the oracle reproduces the reference bit for bit,
    iteration count included."""
    d = np.load(golden("step2d_kat.npz"))
    grid, prm, dt, hn, hc, sf = step2d_case(d, tag)
    Sol = {k: d["%s_in_%s" % (tag, k)].copy() for k in FIELDS}
    p2 = d[tag + "_p2_in"].copy()
    out = n2.impl_part(Sol, p2, hn["S0"], hc, sf, grid, prm, dt)
    assert out["niter"] == int(d[tag + "_niter"])
    np.testing.assert_array_equal(out["rhs"], d[tag + "_rhs"])
    np.testing.assert_array_equal(p2, d[tag + "_p2_out"])
    for k in FIELDS:
        np.testing.assert_array_equal(Sol[k], d["%s_out_%s" % (tag, k)], err_msg=k)


@pytest.mark.parametrize("tag", ["odd", "even", "rk"])
def test_advection_matches_reference_kat(tag):
    """The 2D advection (face mass fluxes, Strang-split sweeps for odd and even
    steps, first-order advect_rk) reproduces the reference bit for bit."""
    from oracle import advection2d as adv
    d = np.load(golden("advect_kat.npz"))
    inx, iny, dt = int(d["meta"][0]), int(d["meta"][1]), float(d["meta"][2])
    grid, prm, _, _, _, hc, sf = cases.rising_bubble(inx=inx, iny=iny)
    hc = dict(hc, rhoY0=d["rhoY0"])          # the reference's background (host exp rounding)
    Sol = {k: d["in_" + k].copy() for k in FIELDS}
    flux = adv.new_flux(grid)
    adv.recompute_advective_fluxes(Sol, flux)
    np.testing.assert_array_equal(flux[0]["rhoY"], d["flux0_rhoY"])
    np.testing.assert_array_equal(flux[1]["rhoY"], d["flux1_rhoY"])
    if tag == "rk":
        pwchi = adv.advect_rk(Sol, flux, 0.5 * dt, grid, prm, hc, sf)
        np.testing.assert_array_equal(pwchi, d["rk_pwchi"])
    else:
        adv.advect(Sol, flux, dt, 1 if tag == "odd" else 0, grid, prm, hc, sf)
    for k in FIELDS:
        np.testing.assert_array_equal(Sol[k], d["%s_%s" % (tag, k)], err_msg=k)


def test_time_step_matches_reference_kat():
    """Two whole time steps of the 64x32 rising bubble (advection, explicit and
    implicit projection halves, Strang sweeps for an even and an odd step):
    the oracle's step reproduces the reference's time_update.do bit for bit."""
    from oracle import advection2d as adv, step2d
    d = np.load(golden("step_kat.npz"))
    grid, prm, Sol_rb, p2_rb, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])   # the reference's background arrays
    Sol = {k: d["in_" + k].copy() for k in FIELDS}
    p2 = d["p2_in"].copy()
    flux = adv.new_flux(grid)
    dt = float(d["meta"][2])
    for step in (0, 1):
        Sol = step2d.time_step(Sol, p2, flux, step, dt, grid, prm, hn, hc, d["S0c"], sf)
        for k in FIELDS:
            np.testing.assert_array_equal(Sol[k], d["s%d_%s" % (step + 1, k)], err_msg="step %d %s" % (step, k))
        np.testing.assert_array_equal(p2, d["s%d_p2" % (step + 1)])


def test_run_to_tout_matches_reference_kat():
    """The loop of time_update.do with the CFL time step: a run with stepmax 4
    reaches tout = 0.1 after three steps (21.69 ms twice, then the CFL step cut
    to tout); the oracle's run reproduces the reference's state bit for bit."""
    from oracle import step2d
    d = np.load(golden("step_kat.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])
    Sol = {k: d["in_" + k].copy() for k in FIELDS}
    p2 = d["p2_in"].copy()
    Sol, t, dts, _ = step2d.run(Sol, p2, 0.0, float(d["meta"][7]), 4, grid, prm, hn, hc, d["S0c"], sf,
                             float(d["meta"][6]))
    assert len(dts) == 3 and t == pytest.approx(float(d["meta"][7]), rel=1e-15)
    for k in FIELDS:
        np.testing.assert_array_equal(Sol[k], d["s4_" + k], err_msg=k)
    np.testing.assert_array_equal(p2, d["s4_p2"])


@pytest.mark.parametrize("case", ["pwp", "wwp"])
@pytest.mark.parametrize("tag", ["odd", "even", "rk"])
def test_advection3d_matches_reference_kat(case, tag):
    """The 3D advection (three face mass fluxes, Strang sweeps with the flips of
    Vars.flip_forward/backward, first-order step) reproduces the reference bit
    for bit for periodic/wall/periodic and wall/wall/periodic boundaries."""
    from oracle import advection3d as a3, proj3d as o3
    d = np.load(golden("advect3d_kat.npz"))
    m = d[case + "_meta"]
    walls = [bool(v) for v in m[3:6]]
    grid = o3.Grid3D(int(m[0]), int(m[1]), int(m[2]), -1.0, 1.0, 0.0, 1.0, -1.0, 1.0,
                     bdry=[n2.WALL if w else n2.PERIODIC for w in walls])
    prm = n2.Params(Msq=float(m[7]), g=float(m[8]), gamm=float(m[9]))
    hc = dict(rhoY0=d[case + "_rhoY0"])
    dt = float(m[6])
    Sol = {k: d["%s_in_%s" % (case, k)].copy() for k in FIELDS}
    flux = a3.new_flux(grid)
    a3.recompute_advective_fluxes(Sol, flux)
    for q in range(3):
        np.testing.assert_array_equal(flux[q]["rhoY"], d["%s_flux%d_rhoY" % (case, q)])
    if tag == "rk":
        pwchi = a3.advect_rk(Sol, flux, 0.5 * dt, grid, prm, hc, lambda y: 1.0)
        np.testing.assert_array_equal(pwchi, d[case + "_rk_pwchi"])
    else:
        a3.advect(Sol, flux, dt, 1 if tag == "odd" else 0, grid, prm, hc, lambda y: 1.0)
    for k in FIELDS:
        np.testing.assert_array_equal(Sol[k], d["%s_%s_%s" % (case, tag, k)], err_msg=k)


def test_oracle_operator_left_null_vector():
    """Seam-consistent vectors: the trapezoid weights annihilate the range.

    For x with equal values on the duplicated periodic seam, the pseudo-
    incompressible operator's output satisfies <w, D A x> = 0 with w the
    trapezoid weights (1/2 on the seam columns) and D = 1/diag_inv.
    """
    rng = np.random.default_rng(3)
    grid = n2.Grid2D(33, 17, -1.0, 1.0, 0.0, 1.0, (n2.PERIODIC, n2.WALL))
    cells = rng.uniform(0.5, 2.0, grid.elem_sc)
    cells[:2] = cells[-4:-2]
    cells[-2:] = cells[2:4]
    wplus = np.stack([cells, cells])
    wcenter = np.zeros(grid.node_isc)
    cor = tuple(np.broadcast_to(v, grid.elem_sc).T.copy() for v in (1.0, 0.9, 0.0, 0.0))
    dinv = n2.precon_diag_prepare(wplus, wcenter, grid.dx, grid.dy)
    op = n2.pack_9pt(wplus, wcenter, cor, dinv, grid)
    x = rng.standard_normal((grid.iny, grid.inx))
    x[:, -1] = x[:, 0]
    y = n2.lap2d_gather(x.reshape(-1), op)
    w = cases.null_weights_2d(grid).T.reshape(-1) / op["diag_inv"]
    assert abs(np.dot(w, y)) < 1e-10 * np.abs(w * y).sum()
    # constants are in the null space
    assert np.abs(n2.lap2d_gather(np.ones(grid.inx * grid.iny), op)).max() < 1e-9


def test_stratified_rhs_is_consistent():
    """The synthetic 2049x1025-type RHS is compatible (small grid for speed)."""
    w = cases.stratified_2d(seed=0, inx=65, iny=33)
    x, info, it = bicgstab_legacy(w["op"], w["b"], 1e-8, 5000)
    assert info == 0
    assert true_relres(w["op"], x, w["b"]) <= 1e-8


def _explicit_case(tag):
    from oracle import nodal2d as n2
    d = np.load(golden("explicit_kat.npz"))
    sc = d[tag + "_scalars"]
    Msq, g, gamm, nonhydro, compressibility, is_comp, dt = sc[:7]
    cor, wind, arakawa = sc[7:10], sc[10:13], int(sc[13])
    grid = n2.Grid2D(64, 32, -1.0, 1.0, 0.0, 1.0, (n2.PERIODIC, n2.WALL))
    prm = n2.Params(Msq=Msq, g=g, gamm=gamm, coriolis=cor, nonhydro=nonhydro, is_compressible=int(is_comp),
                    compressibility=compressibility)
    Sol = {k: d["%s_in_%s" % (tag, k)].copy() for k in ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")}
    hc = {"rhoY0": d[tag + "_rhoY0"]}
    return d, grid, prm, Sol, hc, float(dt), wind, arakawa


@pytest.mark.parametrize("tag", ["a", "b"])
def test_oracle_explicit_parts_match_reference(tag):
    """euler_forward_non_advective and euler_backward_non_advective_expl_part
    (second_projection.py:22-92) against the reference's outputs."""
    from oracle import nodal2d as n2
    d, grid, prm, Sol, hc, dt, wind, arakawa = _explicit_case(tag)
    strat = lambda y: 1.0
    p2 = d[tag + "_p2_in"].copy()
    S = {k: v.copy() for k, v in Sol.items()}
    rhs = n2.euler_forward_non_advective(S, p2, d[tag + "_S0c"], d[tag + "_S0n"], grid, prm, dt, hc, strat,
                                         wind=wind, is_ArakawaKonor=arakawa)
    # bit for bit (same expression order; the box sum uses the reference's fftconvolve)
    for k in S:
        np.testing.assert_array_equal(S[k], d["%s_fw_%s" % (tag, k)], err_msg=k)
    np.testing.assert_array_equal(p2, d[tag + "_fw_p2"])
    np.testing.assert_array_equal(rhs, d[tag + "_fw_rhs"])
    S = {k: v.copy() for k, v in Sol.items()}
    n2.euler_backward_non_advective_expl_part(S, d[tag + "_S0n"], grid, prm, dt, hc, strat, wind=wind)
    for k in S:
        np.testing.assert_array_equal(S[k], d["%s_ex_%s" % (tag, k)], err_msg=k)


def test_oracle_output_loop_matches_reference_full_run():
    """The oracle's output loop (``step2d.run_outputs``: __main__.py:198-393 around
    time_update.do) against the reference's own rising-bubble run
    (``fullrun_kat.npz``, 160x80 cells): theta at t = 0.1 (3 steps, one output
    time) and t = 0.2 (13 steps over eleven output times, so the step index and
    t carry across calls).  Equal to rounding: scipy's inner products come from
    BLAS, whose summation order follows the host's thread count."""
    from oracle import cases, step2d
    d = np.load(golden("fullrun_kat.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble()
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])
    Sol = {k: d["in_" + k].copy() for k in FIELDS}
    p2 = d["p2_in"].copy()
    want = {round(float(t), 3): th for t, th in zip(d["theta_t"], d["theta"]) if t <= 0.2 + 1e-9}
    touts = np.arange(0.0, 1.01, 0.01)[10:21]
    got = {}

    def on_output(t, S, p, step):
        if round(t, 3) in want:
            got[round(t, 3)] = (S["rhoY"] / S["rho"], step)
    step2d.run_outputs(Sol, p2, touts[:1 if len(want) == 1 else 11], 10000, grid, prm, hn, hc, d["S0c"], sf, 1000.0,
                       on_output=on_output)
    assert set(got) == set(want)
    for t, th in want.items():
        mine, step = got[t]
        assert np.abs(mine - th).max() <= 1e-13, (t, np.abs(mine - th).max())
    assert got[0.1][1] == 3


@pytest.mark.parametrize("tag", ["std", "std_cor", "lamb", "lamb_plain"])
def test_oracle_stencil_factory_matches_reference(tag):
    """Both closures of the reference's stencil_9pt_numba_test (laplacian.py:496-543):
    lap2D_gather_new and, with ud.LAMB_BDRY, lap2D_numba_test with the kernel_9pt
    stencil (mirrored y padding), on the reference's own grid/MPV objects
    (stencil_kat.npz): the oracle's packing and operators reproduce them bit for bit."""
    from types import SimpleNamespace as NS
    from oracle import nodal2d as n2
    d = np.load(golden("stencil_kat.npz"))
    m = d[tag + "_meta"]
    g = NS(inx=int(m[0]), iny=int(m[1]), dx=float(m[2]), dy=float(m[3]), x_wall=False, y_wall=True)
    op = n2.pack_9pt(d[tag + "_wplus"], d[tag + "_wcenter"], tuple(d[tag + "_cor%d" % k] for k in range(4)),
                     d[tag + "_diag_inv"], g)
    y = n2.lap2d_lamb(d[tag + "_p"], op) if m[4] else n2.lap2d_gather(d[tag + "_p"], op)
    np.testing.assert_array_equal(y, d[tag + "_y"])
