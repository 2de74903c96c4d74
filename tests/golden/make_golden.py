"""Generate the golden fixtures under tests/golden/ from the pyBELLA reference.

Run in a container where the reference is checked out (it is not needed at
test time; the fixtures are committed):

    python tests/golden/make_golden.py /path/to/pyBELLA [--3d-only]

It imports the reference through ``refshim`` (numba, h5py, ... stubbed; SciPy
``tol=`` keyword restored) and records:

* ``lap2d_kat.npz``   -- ``lap2D_gather_new`` (laplacian.py:546-746) on random
  operands for three grids / boundary combinations, incl. Coriolis cross terms;
* ``lap3d_kat.npz``   -- ``lap3D`` (laplacian.py:898-1026) called directly on
  random operands: four grids (nx == nz) and boundary combinations, Coriolis
  cross terms, the periodic seam overwrite;
* ``diag3d_kat.npz``  -- the 3D branch of ``precon_diag_prepare``;
* ``wall_kat.npz``    -- ``scale_wall_node_values`` for wall/periodic mixes in
  2D and 3D (its index carries over between wall axes);
* ``proj3d_kat.npz``  -- the projection pieces in 3D (boundary data,
  coefficients, divergence, ghost nodes, correction, the explicit part) on two
  small states;
* ``step2d_kat.npz``  -- the whole 2D step on 33x17 states with walls in x and
  y, and with Coriolis in the compressible regime;
* ``advect_kat.npz``  -- the 2D advection (face mass fluxes, Strang-split
  ``advect`` for odd and even steps, ``advect_rk``) on a perturbed 64x32 state;
* ``advect3d_kat.npz`` -- the 3D advection on small 3D states, two boundary mixes;
* ``step_kat.npz``    -- the whole time step (``time_update.do``) of the 64x32
  rising bubble, after one and two steps and a run to tout;
* ``diag_kat.npz``    -- ``precon_diag_prepare`` (laplacian.py:1284-1356);
* ``stencil_kat.npz`` -- the operator factory ``stencil_9pt_numba_test``
  (laplacian.py:496-528) called with the reference's own grid and MPV objects
  on random operands, and its closure applied to a random vector: the
  ``lap2D_gather_new`` branch (periodic x, wall y; with and without Coriolis
  cross terms) and the ``LAMB_BDRY`` branch (``lap2D_numba_test`` with the
  ``kernel_9pt`` stencil, laplacian.py:531-543, 749-868);
* ``pieces_kat.npz``  -- ``divergence_nodes``, ``correction_nodes``,
  ``set_ghostnodes_p2`` and ``set_explicit_boundary_data`` on a random state;
* ``explicit_kat.npz`` -- ``euler_forward_non_advective`` and
  ``euler_backward_non_advective_expl_part`` (second_projection.py:22-92) on
  perturbed rising-bubble states, with and without Coriolis / background wind /
  compressibility;
* ``rising_bubble_step0.npz`` -- inputs and outputs of the two non-trivial
  ``euler_backward_non_advective_impl_part`` calls of the first rising-bubble
  time step (160x80 cells, pseudo-incompressible, tol 1e-10): the full-step
  call (no ``Sol0``) and the next half-step call (with ``Sol0``).
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refshim  # noqa: E402

FIELDS = ["rho", "rhou", "rhov", "rhow", "rhoY", "rhoX"]


def _ud_rising_bubble():
    import utils.user_data as user_data
    import inputs.rising_bubble as rb
    ud = user_data.UserDataInit()
    for k, v in vars(rb.UserData()).items():
        setattr(ud, k, v)
    ud.is_compressible = 0
    ud.compressibility = 0.0
    ud.tol = 1e-10
    ud.coriolis_strength = np.array(ud.coriolis_strength)
    return ud


def lap2d_kat(out):
    import dycore.physics.low_mach.laplacian as lm_lp
    rng = np.random.default_rng(1234)
    cases = [(9, 7, False, True), (12, 10, False, False), (10, 8, True, True)]
    rec = {}
    for ci, (nx, ny, x_wall, y_wall) in enumerate(cases):
        nc = (nx + 1) * (ny + 1)
        hx = rng.uniform(0.5, 2.0, nc)
        hy = rng.uniform(0.5, 2.0, nc)
        hc = rng.uniform(-1.0, 0.0, nx * ny)
        cor = tuple(rng.uniform(-0.5, 1.5, nc) for _ in range(4))
        dinv = rng.uniform(-2.0, -0.5, nx * ny)
        p = rng.standard_normal(nx * ny)
        dx, dy = 0.1 + 0.05 * ci, 0.07 + 0.02 * ci
        y = lm_lp.lap2D_gather_new(p.copy(), nx, ny, (hx, hy, hc), dx, dy, False, x_wall, y_wall,
                                   dinv, cor)
        for k, v in dict(hx=hx, hy=hy, hc=hc, cxx=cor[0], cyy=cor[1], cxy=cor[2], cyx=cor[3],
                         dinv=dinv, p=p, y=y,
                         meta=np.array([nx, ny, int(x_wall), int(y_wall), dx, dy])).items():
            rec["c%d_%s" % (ci, k)] = v
    np.savez_compressed(os.path.join(out, "lap2d_kat.npz"), **rec)


def diag_kat(out):
    import dycore.physics.low_mach.laplacian as lm_lp
    import dycore.utils.options as opts
    rng = np.random.default_rng(99)
    nx, ny = 15, 9
    wplus = rng.uniform(0.5, 2.0, (2, nx + 3, ny + 3))
    wcenter = rng.uniform(-1.0, 0.0, (nx + 2, ny + 2))
    mpv = types.SimpleNamespace(wplus=wplus, wcenter=wcenter)
    node = types.SimpleNamespace(dx=0.1, dy=0.07, dz=1.0, igs=[2, 2, 0])
    elem = types.SimpleNamespace(ndim=2)
    ud = types.SimpleNamespace(bdry_type=[opts.BdryType.PERIODIC, opts.BdryType.WALL, opts.BdryType.WALL])
    d = lm_lp.precon_diag_prepare(mpv, elem, node, ud, None)
    np.savez_compressed(os.path.join(out, "diag_kat.npz"), wplus=wplus, wcenter=wcenter, diag_inv=d,
                        meta=np.array([0.1, 0.07]))


def lap3d_kat(out):
    """``lap3D`` (laplacian.py:898-1026) called directly on random operands.

    The reference's 3D projection glue cannot run (second_projection.py:183-203),
    but ``lap3D`` itself is a pure function of its operands.  Its vector is
    reshaped as (z, y, x) = (nz+2, ny+2, nx+2) while its coefficients are indexed
    (x, y, z), which is consistent only for nx == nz: every case has nx == nz.
    The vector carries the one-node halo; a periodic axis overwrites the halo and
    the first inner node with copies (laplacian.py:927-960), so cases a-c give p
    with the duplicated seam already equal (inner node 0 == inner node n-1) and
    case d gives an unequal seam to record the overwrite.  lap3D zeroes the
    hplus planes of wall axes in place: it gets copies.
    """
    import dycore.physics.low_mach.laplacian as lm_lp
    rng = np.random.default_rng(4242)
    cases = [("a", (7, 5, 7), (True, False, True), 0.3, True),
             ("b", (6, 6, 6), (False, False, False), 0.0, True),
             ("c", (5, 7, 5), (True, True, True), -0.2, True),
             ("d", (6, 4, 6), (True, False, True), 0.25, False)]
    rec = {}
    for tag, (nx, ny, nz), per, corrf, seam in cases:
        shp = (nx + 1, ny + 1, nz + 1)
        hx, hy, hz = (rng.uniform(0.5, 2.0, shp) for _ in range(3))
        hc = rng.uniform(-1.0, 0.0, (nx, ny, nz))
        dinv = rng.uniform(-2.0, -0.5, (nx + 2, ny + 2, nz + 2))    # on the vector's nodes, halo included
        p = rng.standard_normal((nx + 2, ny + 2, nz + 2))
        if seam:
            for axis in range(3):
                if per[axis]:
                    src = [slice(None)] * 3
                    dst = [slice(None)] * 3
                    src[axis], dst[axis] = -2, 1
                    p[tuple(dst)] = p[tuple(src)]
        dx, dy, dz = 0.11, 0.07, 0.09
        y = lm_lp.lap3D(p.reshape(-1).copy(), hx.copy(), hy.copy(), hz.copy(), hc, 1.0 / dx ** 2,
                        1.0 / dy ** 2, 1.0 / dz ** 2, np.array(per), dinv, corrf, 1.0 / dx, 1.0 / dz)
        for k, v in dict(hx=hx, hy=hy, hz=hz, hc=hc, dinv=dinv, p=p, y=np.asarray(y),
                         meta=np.array([nx, ny, nz, *[int(v) for v in per], dx, dy, dz, corrf])).items():
            rec["%s_%s" % (tag, k)] = v
    np.savez_compressed(os.path.join(out, "lap3d_kat.npz"), **rec)


def diag3d_kat(out):
    """3D branch of ``precon_diag_prepare`` (laplacian.py:1284-1356)."""
    import dycore.physics.low_mach.laplacian as lm_lp
    import dycore.utils.options as opts
    rng = np.random.default_rng(98)
    nx, ny, nz = 9, 6, 8
    wplus = rng.uniform(0.5, 2.0, (3, nx + 1, ny + 1, nz + 1))
    wcenter = rng.uniform(-1.0, 0.0, (nx, ny, nz))
    mpv = types.SimpleNamespace(wplus=wplus, wcenter=wcenter)
    node = types.SimpleNamespace(dx=0.1, dy=0.07, dz=0.13, igs=[2, 2, 2])
    elem = types.SimpleNamespace(ndim=3)
    ud = types.SimpleNamespace(bdry_type=[opts.BdryType.PERIODIC, opts.BdryType.WALL, opts.BdryType.PERIODIC])
    d = lm_lp.precon_diag_prepare(mpv, elem, node, ud, None)
    np.savez_compressed(os.path.join(out, "diag3d_kat.npz"), wplus=wplus, wcenter=wcenter, diag_inv=d,
                        meta=np.array([0.1, 0.07, 0.13]))


def wall_kat(out):
    """``scale_wall_node_values`` (second_projection.py:433-474) on random node.isc
    arrays for every wall/periodic mix in 2D and several in 3D."""
    import dycore.physics.low_mach.second_projection as lm_sp
    import dycore.utils.options as opts
    W, P = opts.BdryType.WALL, opts.BdryType.PERIODIC
    rng = np.random.default_rng(5)
    rec = {}
    cases = [("ww", (W, W), (9, 7)), ("pw", (P, W), (9, 7)), ("wp", (W, P), (8, 9)),
             ("pwp", (P, W, P), (8, 7, 9)), ("www", (W, W, W), (8, 7, 9)), ("wwp", (W, W, P), (7, 8, 6)),
             ("pww", (P, W, W), (7, 8, 6))]
    for tag, bt, shp in cases:
        a = rng.uniform(0.5, 1.5, shp)
        rec[tag + "_in"] = a.copy()
        node = types.SimpleNamespace(ndim=len(shp), igs=[2] * len(shp))
        for f, name in ((0.5, "half"), (2.0, "two")):
            b = a.copy()
            lm_sp.scale_wall_node_values(b, node, types.SimpleNamespace(bdry_type=list(bt)), f)
            rec["%s_%s" % (tag, name)] = b
        rec[tag + "_walls"] = np.array([int(v == W) for v in bt])
    np.savez_compressed(os.path.join(out, "wall_kat.npz"), **rec)


def proj3d_kat(out):
    """The reference's projection pieces on small 3D states (they are
    dimension-generic; only the step's glue is broken in 3D).

    Case a: periodic x / wall y / periodic z, no Coriolis, pseudo-incompressible.
    Case b: wall x / wall y / periodic z, Coriolis, compressible ghost cells.
    The state is the rising bubble's hydrostatic background in 3D with seeded
    perturbations; each piece runs on a copy of the state left by the previous
    one, as in the projection step."""
    import copy
    import dycore.discretisation.grid as dis_grid
    import dycore.utils.variable as var
    import dycore.physics.low_mach.mpv as lm_var
    import dycore.physics.gas_dynamics.thermodynamic as gd_thermodynamics
    import dycore.physics.low_mach.second_projection as lm_sp
    import dycore.physics.hydrostatics as hydrostatic
    import dycore.utils.boundary as bdry
    import dycore.utils.options as opts
    W, P = opts.BdryType.WALL, opts.BdryType.PERIODIC
    rec = {}
    cases = [("a", (P, W, P), (0.0, 0.0, 0.0), 0, 0.01, 71),
             ("b", (W, W, P), (3.0, 2.0, 1.0), 1, 0.05, 72)]
    for tag, bt, cor, is_comp, dt, seed in cases:
        rng = np.random.default_rng(seed)
        ud = _ud_rising_bubble()
        ud.inx, ud.iny, ud.inz = 9, 7, 8
        ud.zmin, ud.zmax = -1.0, 1.0
        ud.bdry_type = np.array(list(bt))
        ud.coriolis_strength = np.array(cor)
        ud.is_compressible = is_comp
        elem, node = dis_grid.grid_init(ud)
        ud.nonhydrostasy = 1.0
        Sol = var.Vars(elem.sc, ud)
        th = gd_thermodynamics.init(ud)
        mpv = lm_var.MPV(elem, node, ud)
        hydrostatic.state(mpv, elem, node, th, ud)
        rhoY = np.broadcast_to(mpv.HydroState.rhoY0.reshape(1, -1, 1), elem.sc)
        yy = np.broadcast_to(elem.y.reshape(1, -1, 1), elem.sc)
        Sol.rhoY[...] = rhoY * (1.0 + 0.001 * rng.standard_normal(elem.sc))
        Sol.rho[...] = rhoY / ud.stratification(yy) * (1.0 + 0.01 * rng.standard_normal(elem.sc))
        for k in ("rhou", "rhov", "rhow", "rhoX"):
            getattr(Sol, k)[...] = 0.01 * rng.standard_normal(elem.sc)
        for k in FIELDS:
            rec["%s_in_%s" % (tag, k)] = np.copy(getattr(Sol, k))
        bdry.set_explicit_boundary_data(Sol, elem, ud, th, mpv)
        for k in FIELDS:
            rec["%s_bd_%s" % (tag, k)] = np.copy(getattr(Sol, k))
        S = copy.deepcopy(Sol)
        lm_sp.operator_coefficients_nodes(elem, node, S, mpv, ud, th, dt)
        rec[tag + "_wplus"] = np.copy(mpv.wplus)
        rec[tag + "_wcenter"] = np.copy(mpv.wcenter)
        rhs = lm_sp.divergence_nodes(np.zeros(node.sc), elem, node, S, ud)
        rec[tag + "_div"] = np.copy(rhs)
        for k in ("rhou", "rhov", "rhow"):
            rec["%s_dv_%s" % (tag, k)] = np.copy(getattr(S, k))
        p = rng.standard_normal(node.sc)
        rec[tag + "_p"] = np.copy(p)
        q = np.copy(p)
        bdry.set_ghostnodes_p2(q, node, ud)
        rec[tag + "_gn"] = q
        S = copy.deepcopy(Sol)
        lm_sp.correction_nodes(S, elem, node, mpv, q, dt, ud, th, 1)
        for k in FIELDS:
            rec["%s_cr_%s" % (tag, k)] = np.copy(getattr(S, k))
        # euler_backward_non_advective_expl_part (dimension-generic), case b with background wind
        if tag == "b":
            ud.u_wind_speed, ud.v_wind_speed, ud.w_wind_speed = 0.5, 0.0, 0.2
        S = copy.deepcopy(Sol)
        lm_sp.euler_backward_non_advective_expl_part(S, mpv, elem, dt, ud, th)
        for k in FIELDS:
            rec["%s_xp_%s" % (tag, k)] = np.copy(getattr(S, k))
        rec[tag + "_wind"] = np.array([ud.u_wind_speed, ud.v_wind_speed, ud.w_wind_speed])
        rec[tag + "_S0n"] = np.copy(mpv.HydroState_n.S0)
        rec[tag + "_rhoY0"] = np.copy(mpv.HydroState.rhoY0)
        rec[tag + "_strat_inv"] = np.array([1.0 / ud.stratification(y) for y in elem.y])
        rec[tag + "_meta"] = np.array([ud.inx, ud.iny, ud.inz, int(bt[0] == W), int(bt[1] == W), int(bt[2] == W),
                                       node.dx, node.dy, node.dz, dt, ud.Msq, ud.gravity_strength[1], th.gamm,
                                       ud.nonhydrostasy, ud.compressibility, is_comp, *cor])
    np.savez_compressed(os.path.join(out, "proj3d_kat.npz"), **rec)


def _rb_setup():
    import dycore.discretisation.grid as dis_grid
    import dycore.utils.variable as var
    import dycore.physics.low_mach.mpv as lm_var
    import dycore.physics.gas_dynamics.thermodynamic as gd_thermodynamics
    import inputs.rising_bubble as rb
    ud = _ud_rising_bubble()
    elem, node = dis_grid.grid_init(ud)
    Sol = var.Vars(elem.sc, ud)
    th = gd_thermodynamics.init(ud)
    mpv = lm_var.MPV(elem, node, ud)
    Sol = rb.sol_init(Sol, mpv, elem, node, th, ud)
    ud.nonhydrostasy = 1.0
    return ud, elem, node, Sol, th, mpv


def pieces_kat(out):
    """Reference helpers on a random perturbation of a small rising-bubble state."""
    import dycore.discretisation.grid as dis_grid
    import dycore.utils.variable as var
    import dycore.physics.low_mach.mpv as lm_var
    import dycore.physics.gas_dynamics.thermodynamic as gd_thermodynamics
    import dycore.physics.low_mach.second_projection as lm_sp
    import dycore.utils.boundary as bdry
    import inputs.rising_bubble as rb
    rng = np.random.default_rng(7)
    ud = _ud_rising_bubble()
    ud.inx, ud.iny = 17, 11
    elem, node = dis_grid.grid_init(ud)
    Sol = var.Vars(elem.sc, ud)
    th = gd_thermodynamics.init(ud)
    mpv = lm_var.MPV(elem, node, ud)
    Sol = rb.sol_init(Sol, mpv, elem, node, th, ud)
    ud.nonhydrostasy = 1.0
    for k in ("rhou", "rhov", "rhoX"):
        setattr(Sol, k, 0.01 * rng.standard_normal(elem.sc[:2]))
    Sol.rho = Sol.rho * (1.0 + 0.01 * rng.standard_normal(elem.sc[:2]))
    rec = {("in_" + k): np.copy(getattr(Sol, k)) for k in FIELDS}
    p = rng.standard_normal(node.sc[:2])
    rec["p"] = np.copy(p)
    dt = 0.01
    # set_explicit_boundary_data
    bdry.set_explicit_boundary_data(Sol, elem, ud, th, mpv)
    for k in FIELDS:
        rec["bd_" + k] = np.copy(getattr(Sol, k))
    # divergence_nodes (mutates ghost rows of the momenta)
    rhs = np.zeros(node.isc[:2])
    rhs = lm_sp.divergence_nodes(rhs, elem, node, Sol, ud)
    rec["div"] = np.copy(rhs)
    for k in FIELDS:
        rec["dv_" + k] = np.copy(getattr(Sol, k))
    # correction_nodes with updt_chi = 1
    lm_sp.correction_nodes(Sol, elem, node, mpv, p, dt, ud, th, 1)
    for k in FIELDS:
        rec["cr_" + k] = np.copy(getattr(Sol, k))
    # ghost nodes, periodic x / wall y and wall x / periodic y
    q = np.copy(p)
    bdry.set_ghostnodes_p2(q, node, ud)
    rec["gn_pw"] = q
    import dycore.utils.options as opts
    ud2 = types.SimpleNamespace(bdry_type=[opts.BdryType.WALL, opts.BdryType.PERIODIC, opts.BdryType.WALL])
    q2 = np.copy(p)
    bdry.set_ghostnodes_p2(q2, node, ud2)
    rec["gn_wp"] = q2
    rec["meta"] = np.array([ud.inx, ud.iny, dt])
    np.savez_compressed(os.path.join(out, "pieces_kat.npz"), **rec)


def explicit_kat(out):
    """The explicit parts of the projection on perturbed 64x32 rising-bubble states."""
    import dycore.physics.low_mach.second_projection as lm_sp
    rec = {}
    cases = [("a", dict()),
             ("b", dict(coriolis=(0.3, 0.2, 0.1), wind=(0.5, 0.0, 0.2), compressibility=1.0))]
    for tag, opt in cases:
        rng = np.random.default_rng(11 if tag == "a" else 12)
        ud, elem, node, Sol, th, mpv = _rb_setup_sized(64, 32)
        if "coriolis" in opt:
            ud.coriolis_strength = np.array(opt["coriolis"])
            ud.u_wind_speed, ud.v_wind_speed, ud.w_wind_speed = opt["wind"]
            ud.compressibility = opt["compressibility"]
        for k in ("rhou", "rhov", "rhow", "rhoX"):
            setattr(Sol, k, getattr(Sol, k) + 0.01 * rng.standard_normal(elem.sc[:2]))
        Sol.rho = Sol.rho * (1.0 + 0.01 * rng.standard_normal(elem.sc[:2]))
        Sol.rhoY = Sol.rhoY * (1.0 + 0.001 * rng.standard_normal(elem.sc[:2]))
        mpv.p2_nodes[...] = 0.1 * rng.standard_normal(node.sc[:2])
        dt = 0.005
        rec[tag + "_scalars"] = np.array([ud.Msq, ud.gravity_strength[1], th.gamm, ud.nonhydrostasy,
                                          ud.compressibility, ud.is_compressible, dt,
                                          *ud.coriolis_strength, ud.u_wind_speed, ud.v_wind_speed,
                                          ud.w_wind_speed, getattr(ud, "is_ArakawaKonor", 0)])
        rec[tag + "_S0c"] = np.copy(mpv.HydroState.get_S0c(elem))
        rec[tag + "_S0n"] = np.copy(mpv.HydroState_n.S0)
        rec[tag + "_rhoY0"] = np.copy(mpv.HydroState.rhoY0)
        rec[tag + "_strat_inv"] = np.array([1.0 / ud.stratification(y) for y in elem.y])
        for k in FIELDS:
            rec[tag + "_in_" + k] = np.copy(getattr(Sol, k))
        rec[tag + "_p2_in"] = np.copy(mpv.p2_nodes)
        # euler_forward_non_advective on a copy of the state
        import copy
        Sol_f, mpv_f = copy.deepcopy(Sol), copy.deepcopy(mpv)
        lm_sp.euler_forward_non_advective(Sol_f, mpv_f, elem, node, dt, ud, th)
        for k in FIELDS:
            rec[tag + "_fw_" + k] = np.copy(getattr(Sol_f, k))
        rec[tag + "_fw_p2"] = np.copy(mpv_f.p2_nodes)
        rec[tag + "_fw_rhs"] = np.copy(mpv_f.rhs)
        # euler_backward_non_advective_expl_part on another copy
        Sol_e, mpv_e = copy.deepcopy(Sol), copy.deepcopy(mpv)
        lm_sp.euler_backward_non_advective_expl_part(Sol_e, mpv_e, elem, dt, ud, th)
        for k in FIELDS:
            rec[tag + "_ex_" + k] = np.copy(getattr(Sol_e, k))
    np.savez_compressed(os.path.join(out, "explicit_kat.npz"), **rec)


def _rb_setup_sized(inx, iny):
    import dycore.discretisation.grid as dis_grid
    import dycore.utils.variable as var
    import dycore.physics.low_mach.mpv as lm_var
    import dycore.physics.gas_dynamics.thermodynamic as gd_thermodynamics
    import inputs.rising_bubble as rb
    ud = _ud_rising_bubble()
    ud.inx, ud.iny = inx, iny
    elem, node = dis_grid.grid_init(ud)
    Sol = var.Vars(elem.sc, ud)
    th = gd_thermodynamics.init(ud)
    mpv = lm_var.MPV(elem, node, ud)
    Sol = rb.sol_init(Sol, mpv, elem, node, th, ud)
    ud.nonhydrostasy = 1.0
    return ud, elem, node, Sol, th, mpv


def step2d_kat(out):
    """The reference's whole 2D projection step (impl_part) on two small states
    the rising-bubble fixture does not cover, both in the compressible regime
    (hcenter != 0): walls in x and y; and periodic x with Coriolis (cross
    terms).  33x17 nodes, seeded momenta, tol 1e-10.  (With walls in x the
    pseudo-incompressible step does not converge in the reference: its wall
    padding keeps rhou symmetric and negates rhov, boundary.py:161-166, so the
    divergence is not in the range of the singular operator.)"""
    import dycore.physics.low_mach.second_projection as lm_sp
    import dycore.utils.options as opts
    rec = {}
    cases = [("ww", opts.BdryType.WALL, (0.0, 0.0, 0.0), 1, 1.0, 21),
             ("cor", opts.BdryType.PERIODIC, (3.0, 2.0, 1.0), 1, 1.0, 22)]
    for tag, xb, cor, is_comp, comp, seed in cases:
        rng = np.random.default_rng(seed)
        ud, elem, node, Sol, th, mpv = _rb_setup_sized(33, 17)
        ud.bdry_type[0] = xb
        ud.coriolis_strength = np.array(cor)
        ud.is_compressible, ud.compressibility = is_comp, comp
        for k in ("rhou", "rhov", "rhow"):
            setattr(Sol, k, getattr(Sol, k) + 0.05 * Sol.rho * rng.standard_normal(elem.sc[:2]))
        mpv.p2_nodes[...] = 0.01 * rng.standard_normal(node.sc[:2])
        import dycore.utils.boundary as bdry
        bdry.set_explicit_boundary_data(Sol, elem, ud, th, mpv)
        dt = 0.01
        for k in FIELDS:
            rec["%s_in_%s" % (tag, k)] = np.copy(getattr(Sol, k))
        rec[tag + "_p2_in"] = np.copy(mpv.p2_nodes)
        n0 = lm_sp.total_iter
        lm_sp.euler_backward_non_advective_impl_part(Sol, mpv, elem, node, ud, th, 0.0, dt, 1.0)
        rec[tag + "_niter"] = np.array(lm_sp.total_iter - n0)
        for k in FIELDS:
            rec["%s_out_%s" % (tag, k)] = np.copy(getattr(Sol, k))
        rec[tag + "_p2_out"] = np.copy(mpv.p2_nodes)
        rec[tag + "_rhs"] = np.copy(mpv.rhs)
        rec[tag + "_S0n"] = np.copy(mpv.HydroState_n.S0)
        rec[tag + "_rhoY0"] = np.copy(mpv.HydroState.rhoY0)
        rec[tag + "_meta"] = np.array([33, 17, int(xb == opts.BdryType.WALL), dt, ud.Msq, ud.gravity_strength[1],
                                       th.gamm, is_comp, comp, *cor])
        print("step2d %s: %d iterations" % (tag, int(rec[tag + "_niter"])), flush=True)
    np.savez_compressed(os.path.join(out, "step2d_kat.npz"), **rec)


def advect_kat(out):
    """The reference's 2D advection on a perturbed 64x32 rising-bubble state:
    the face mass fluxes (recompute_advective_fluxes), the Strang-split
    ``advect`` for an odd and an even step, and the first-order ``advect_rk``,
    each from the same state and freshly computed fluxes."""
    import copy
    import dycore.utils.variable as var
    import dycore.physics.gas_dynamics.explicit as gd_explicit
    import dycore.physics.gas_dynamics.numerical_flux as gd_flux
    rng = np.random.default_rng(31)
    ud, elem, node, Sol, th, mpv = _rb_setup_sized(64, 32)
    for k in ("rhou", "rhov", "rhow"):
        setattr(Sol, k, getattr(Sol, k) + 0.1 * Sol.rho * rng.standard_normal(elem.sc[:2]))
    Sol.rhoX = Sol.rhoX + 0.01 * Sol.rho * rng.standard_normal(elem.sc[:2])
    import dycore.utils.boundary as bdry
    bdry.set_explicit_boundary_data(Sol, elem, ud, th, mpv)
    rec = {("in_" + k): np.copy(getattr(Sol, k)) for k in FIELDS}
    dt = 0.01
    for tag, call in (("odd", lambda S, f: gd_explicit.advect(S, f, dt, elem, 1, ud, th, mpv, node, "x")),
                      ("even", lambda S, f: gd_explicit.advect(S, f, dt, elem, 0, ud, th, mpv, node, "x")),
                      ("rk", lambda S, f: gd_explicit.advect_rk(S, f, 0.5 * dt, elem, 0, ud, th, mpv, node, "x"))):
        S = copy.deepcopy(Sol)
        flux = np.empty((3), dtype=object)
        flux[0] = var.States(elem.sfx, ud)
        flux[1] = var.States(elem.sfy, ud)
        gd_flux.recompute_advective_fluxes(flux, S)
        if tag == "odd":
            rec["flux0_rhoY"] = np.copy(flux[0].rhoY)
            rec["flux1_rhoY"] = np.copy(flux[1].rhoY)
        call(S, flux)
        for k in FIELDS:
            rec["%s_%s" % (tag, k)] = np.copy(getattr(S, k))
        if tag == "rk":
            rec["rk_pwchi"] = np.copy(S.pwchi)
    rec["meta"] = np.array([64, 32, dt, ud.Msq, ud.gravity_strength[1], th.gamm])
    rec["S0n"] = np.copy(mpv.HydroState_n.S0)
    rec["rhoY0"] = np.copy(mpv.HydroState.rhoY0)
    np.savez_compressed(os.path.join(out, "advect_kat.npz"), **rec)


def advect3d_kat(out):
    """The reference's 3D advection (dimension-generic in the reference): face
    mass fluxes, Strang-split ``advect`` for an odd and an even step and
    ``advect_rk``, on the 3D hydrostatic state with seeded perturbations, for
    periodic/wall/periodic and wall/wall/periodic boundaries."""
    import copy
    import dycore.discretisation.grid as dis_grid
    import dycore.utils.variable as var
    import dycore.physics.low_mach.mpv as lm_var
    import dycore.physics.gas_dynamics.thermodynamic as gd_thermodynamics
    import dycore.physics.hydrostatics as hydrostatic
    import dycore.physics.gas_dynamics.explicit as gd_explicit
    import dycore.physics.gas_dynamics.numerical_flux as gd_flux
    import dycore.utils.boundary as bdry
    import dycore.utils.options as opts
    W, P = opts.BdryType.WALL, opts.BdryType.PERIODIC
    rec = {}
    for case, bt, seed in (("pwp", (P, W, P), 41), ("wwp", (W, W, P), 42)):
        rng = np.random.default_rng(seed)
        ud = _ud_rising_bubble()
        ud.inx, ud.iny, ud.inz = 9, 7, 8
        ud.zmin, ud.zmax = -1.0, 1.0
        ud.bdry_type = np.array(list(bt))
        elem, node = dis_grid.grid_init(ud)
        ud.nonhydrostasy = 1.0
        Sol = var.Vars(elem.sc, ud)
        th = gd_thermodynamics.init(ud)
        mpv = lm_var.MPV(elem, node, ud)
        hydrostatic.state(mpv, elem, node, th, ud)
        rhoY = np.broadcast_to(mpv.HydroState.rhoY0.reshape(1, -1, 1), elem.sc)
        Sol.rhoY[...] = rhoY
        Sol.rho[...] = rhoY * (1.0 + 0.01 * rng.standard_normal(elem.sc))
        for k in ("rhou", "rhov", "rhow", "rhoX"):
            getattr(Sol, k)[...] = 0.1 * Sol.rho * rng.standard_normal(elem.sc)
        bdry.set_explicit_boundary_data(Sol, elem, ud, th, mpv)
        for k in FIELDS:
            rec["%s_in_%s" % (case, k)] = np.copy(getattr(Sol, k))
        dt = 0.01
        for tag, call in (("odd", lambda S, f: gd_explicit.advect(S, f, dt, elem, 1, ud, th, mpv, node, "x")),
                          ("even", lambda S, f: gd_explicit.advect(S, f, dt, elem, 0, ud, th, mpv, node, "x")),
                          ("rk", lambda S, f: gd_explicit.advect_rk(S, f, 0.5 * dt, elem, 0, ud, th, mpv, node,
                                                                    "x"))):
            S = copy.deepcopy(Sol)
            flux = np.empty((3), dtype=object)
            flux[0] = var.States(elem.sfx, ud)
            flux[1] = var.States(elem.sfy, ud)
            flux[2] = var.States(elem.sfz, ud)
            gd_flux.recompute_advective_fluxes(flux, S)
            if tag == "odd":
                for q in range(3):
                    rec["%s_flux%d_rhoY" % (case, q)] = np.copy(flux[q].rhoY)
            call(S, flux)
            for k in FIELDS:
                rec["%s_%s_%s" % (case, tag, k)] = np.copy(getattr(S, k))
            if tag == "rk":
                rec[case + "_rk_pwchi"] = np.copy(S.pwchi)
        rec[case + "_rhoY0"] = np.copy(mpv.HydroState.rhoY0)
        rec[case + "_meta"] = np.array([9, 7, 8, int(bt[0] == W), int(bt[1] == W), int(bt[2] == W), dt,
                                        ud.Msq, ud.gravity_strength[1], th.gamm])
    np.savez_compressed(os.path.join(out, "advect3d_kat.npz"), **rec)


def step_kat(out):
    """The reference's whole time step (time_update.do, time_update.py:129-708) on
    the 64x32 rising bubble: the state after one and two steps (fixed dt =
    21.69 / t_ref, 'CFLfixed') and after a run with stepmax 4, which reaches
    tout[0] = 0.1 after three steps (the CFL step of the third is cut to tout)."""
    import dycore.discretisation.time_update as dis_time_update
    import dycore.utils.variable as var
    from data_assimilation import blending as da_blending
    rec = {}
    for nsteps in (1, 2, 4):
        ud, elem, node, Sol, th, mpv = _rb_setup_sized(64, 32)
        if nsteps == 1:
            for k in FIELDS:
                rec["in_" + k] = np.copy(getattr(Sol, k))
            rec["p2_in"] = np.copy(mpv.p2_nodes)
            rec["S0n"] = np.copy(mpv.HydroState_n.S0)
            rec["rhoY0"] = np.copy(mpv.HydroState.rhoY0)
            rec["S0c"] = np.copy(mpv.HydroState.get_S0c(elem))
        ud.stepmax = nsteps
        flux = np.empty((3), dtype=object)
        flux[0] = var.States(elem.sfx, ud)
        flux[1] = var.States(elem.sfy, ud)
        ret = dis_time_update.do(Sol, flux, mpv, 0.0, ud.tout[0], ud, elem, node, [0, 0], th,
                                 da_blending.Blend(ud), None, False)
        S, m = ret[0], ret[2]
        for k in FIELDS:
            rec["s%d_%s" % (nsteps, k)] = np.copy(getattr(S, k))
        rec["s%d_p2" % nsteps] = np.copy(m.p2_nodes)
        print("step_kat: %d step(s) done" % nsteps, flush=True)
    rec["meta"] = np.array([64, 32, 21.69 / ud.t_ref, ud.Msq, ud.gravity_strength[1], th.gamm, ud.t_ref,
                            ud.tout[0]])
    np.savez_compressed(os.path.join(out, "step_kat.npz"), **rec)


def rising_bubble_step0(out):
    import dycore.discretisation.time_update as dis_time_update
    import dycore.physics.low_mach.second_projection as lm_sp
    import dycore.utils.variable as var
    from data_assimilation import blending as da_blending
    ud, elem, node, Sol, th, mpv = _rb_setup()
    flux = np.empty((3), dtype=object)
    flux[0] = var.States(elem.sfx, ud)
    flux[1] = var.States(elem.sfy, ud)
    bld = da_blending.Blend(ud)
    calls = []
    orig = lm_sp.euler_backward_non_advective_impl_part

    def wrapped(Sol, mpv, elem, node, ud, th, t, dt, alpha_diff, Sol0=None, writer=None,
                label=None, debug=False):
        rec = dict(dt=dt, sol_in={k: np.copy(getattr(Sol, k)) for k in FIELDS},
                   sol0_in=None if Sol0 is None else {k: np.copy(getattr(Sol0, k)) for k in FIELDS},
                   p2_in=np.copy(mpv.p2_nodes))
        n0 = lm_sp.total_iter
        orig(Sol, mpv, elem, node, ud, th, t, dt, alpha_diff, Sol0=Sol0, writer=writer, label=label,
             debug=debug)
        rec["niter"] = lm_sp.total_iter - n0
        rec["sol_out"] = {k: np.copy(getattr(Sol, k)) for k in FIELDS}
        rec["p2_out"] = np.copy(mpv.p2_nodes)
        rec["rhs"] = np.copy(mpv.rhs)
        calls.append(rec)
        print("impl_part call %d: dt=%g niter=%d" % (len(calls), dt, rec["niter"]), flush=True)

    lm_sp.euler_backward_non_advective_impl_part = wrapped
    dis_time_update.do(Sol, flux, mpv, 0.0, ud.tout[0], ud, elem, node, [0, 0], th, bld, None, False)
    rec = {}
    for tag, ci in (("full", 1), ("half", 2)):
        c = calls[ci]
        rec[tag + "_dt"] = np.array(c["dt"])
        rec[tag + "_niter"] = np.array(c["niter"])
        rec[tag + "_p2_in"] = c["p2_in"]
        rec[tag + "_p2_out"] = c["p2_out"]
        rec[tag + "_rhs"] = c["rhs"]
        for k in FIELDS:
            rec[tag + "_in_" + k] = c["sol_in"][k]
            rec[tag + "_out_" + k] = c["sol_out"][k]
            if c["sol0_in"] is not None:
                rec[tag + "_sol0_" + k] = c["sol0_in"][k]
    rec["hydro_n_S0"] = np.copy(mpv.HydroState_n.S0)
    rec["hydro_c_rhoY0"] = np.copy(mpv.HydroState.rhoY0)
    rec["scalars"] = np.array([ud.Msq, ud.gravity_strength[1], th.gamm])
    np.savez_compressed(os.path.join(out, "rising_bubble_step0.npz"), **rec)


def stencil_kat(out):
    import dycore.discretisation.grid as dis_grid
    import dycore.physics.low_mach.laplacian as lm_lp
    import dycore.physics.low_mach.mpv as lm_var
    rec = {}
    rng = np.random.default_rng(23)
    for tag, lamb, cor, comp in (("std", False, False, False), ("std_cor", False, True, True),
                                 ("lamb", True, True, True), ("lamb_plain", True, False, False)):
        ud = _ud_rising_bubble()
        ud.inx, ud.iny = 33, 17
        elem, node = dis_grid.grid_init(ud)
        mpv = lm_var.MPV(elem, node, ud)
        if lamb:
            ud.LAMB_BDRY = False              # the reference tests hasattr (test_lamb_wave.py:87)
        mpv.wplus[...] = 0.5 + rng.random(mpv.wplus.shape)
        mpv.wcenter[...] = -(0.5 + rng.random(mpv.wcenter.shape)) if comp else 0.0
        csh = (elem.sc[1], elem.sc[0])        # transposed cell arrays (second_projection.py:651)
        coriolis = (1.0 + 0.1 * rng.random(csh), 0.8 + 0.1 * rng.random(csh),
                    0.1 * rng.standard_normal(csh) if cor else np.zeros(csh),
                    0.1 * rng.standard_normal(csh) if cor else np.zeros(csh))
        diag_inv = -(0.5 + rng.random(node.isc[:2]))     # 2D, as precon_diag_prepare returns it
        f = lm_lp.stencil_9pt_numba_test(mpv, node, coriolis, diag_inv, ud)
        p = rng.standard_normal(node.iicx * node.iicy)
        y = f(p.copy())
        rec[tag + "_wplus"] = np.copy(mpv.wplus)
        rec[tag + "_wcenter"] = np.copy(mpv.wcenter)
        for k in range(4):
            rec[tag + "_cor%d" % k] = np.copy(coriolis[k])
        rec[tag + "_diag_inv"] = np.copy(diag_inv)
        rec[tag + "_p"] = p
        rec[tag + "_y"] = np.copy(y)
        rec[tag + "_meta"] = np.array([node.iicx, node.iicy, node.dx, node.dy, int(lamb)])
        print("stencil_kat: %s done" % tag, flush=True)
    np.savez_compressed(os.path.join(out, "stencil_kat.npz"), **rec)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if not args:
        raise SystemExit("usage: make_golden.py REFERENCE_ROOT [--3d-only | --explicit-only | --stencil-only]")
    ref = args[0]
    refshim.install(ref)
    out = HERE
    if "--stencil-only" in sys.argv:
        stencil_kat(out)
        return
    lap3d_kat(out)
    diag3d_kat(out)
    wall_kat(out)
    proj3d_kat(out)
    step2d_kat(out)
    advect_kat(out)
    advect3d_kat(out)
    step_kat(out)
    if "--3d-only" in sys.argv:
        print("fixtures written to", out)
        return
    lap2d_kat(out)
    diag_kat(out)
    pieces_kat(out)
    explicit_kat(out)
    stencil_kat(out)
    if "--explicit-only" not in sys.argv:
        rising_bubble_step0(out)
    print("fixtures written to", out)


if __name__ == "__main__":
    main()
