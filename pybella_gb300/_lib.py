"""ctypes binding of libbella_gb300.so (the C ABI declared in include/bella.h).

The library is the only compute path: if it is missing this module raises,
it never falls back to a CPU implementation.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbella_gb300.so")

BELLA_OK = 0
BELLA_MAXITER = 1
BELLA_BREAKDOWN = 2
BELLA_NONFINITE = 3
BELLA_TIMEOUT = 4
BELLA_EINVAL = -1
BELLA_ECUDA = -2
BELLA_ENOOP = -3
BELLA_Y_MIRROR = 2      # bella_op2d.y_wall: the mirrored y boundary of the LAMB_BDRY stencil

_dp = ctypes.c_void_p


class Op2D(ctypes.Structure):
    """``bella_op2d``: reference-packed 2D operands (device pointers)."""
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("x_wall", ctypes.c_int), ("y_wall", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("hplusx", _dp), ("hplusy", _dp), ("hcenter", _dp),
                ("cxx", _dp), ("cyy", _dp), ("cxy", _dp), ("cyx", _dp),
                ("diag_inv", _dp)]


class Op3D(ctypes.Structure):
    """``bella_op3d``: 3D 27-point operands (device pointers, C order, z fastest)."""
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("x_wall", ctypes.c_int), ("y_wall", ctypes.c_int), ("z_wall", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("corrf", ctypes.c_double),
                ("hplusx", _dp), ("hplusy", _dp), ("hplusz", _dp), ("hcenter", _dp), ("diag_inv", _dp)]


class Proj2D(ctypes.Structure):
    """``bella_proj2d``: device arrays of one 2D projection (reference layout)."""
    _fields_ = [("inx", ctypes.c_int), ("iny", ctypes.c_int), ("x_wall", ctypes.c_int), ("y_wall", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dt", ctypes.c_double),
                ("Msq", ctypes.c_double), ("g", ctypes.c_double), ("gamm", ctypes.c_double),
                ("nonhydro", ctypes.c_double), ("compressibility", ctypes.c_double),
                ("coriolis", ctypes.c_double * 3), ("is_compressible", ctypes.c_int), ("precond", ctypes.c_int)] + \
        [(k, _dp) for k in ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX",
                            "rho0", "rhou0", "rhov0", "rhow0", "rhoY0", "rhoX0",
                            "p2", "hydro_rhoY0", "S0n", "strat_inv", "rhs_out")]


class Proj3D(ctypes.Structure):
    """``bella_proj3d``: device arrays of one 3D projection (reference layout)."""
    _fields_ = [("inx", ctypes.c_int), ("iny", ctypes.c_int), ("inz", ctypes.c_int),
                ("x_wall", ctypes.c_int), ("y_wall", ctypes.c_int), ("z_wall", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
                ("Msq", ctypes.c_double), ("g", ctypes.c_double), ("gamm", ctypes.c_double),
                ("nonhydro", ctypes.c_double), ("compressibility", ctypes.c_double),
                ("coriolis", ctypes.c_double * 3), ("is_compressible", ctypes.c_int), ("precond", ctypes.c_int)] + \
        [(k, _dp) for k in ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX",
                            "rho0", "rhou0", "rhov0", "rhow0", "rhoY0", "rhoX0",
                            "p2", "hydro_rhoY0", "S0n", "strat_inv", "rhs_out")] + \
        [("div_sign_2d", ctypes.c_int)]


class Adv2D(ctypes.Structure):
    """``bella_adv2d``: device arrays of the 2D advection (reference layout)."""
    _fields_ = [("inx", ctypes.c_int), ("iny", ctypes.c_int), ("x_wall", ctypes.c_int), ("y_wall", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("g", ctypes.c_double), ("gamm", ctypes.c_double),
                ("is_compressible", ctypes.c_int), ("pad_", ctypes.c_int)] + \
        [(k, _dp) for k in ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")] + \
        [("fx", _dp * 6), ("fy", _dp * 6), ("hydro_rhoY0", _dp), ("strat_inv", _dp), ("pwchi", _dp)]


class Adv3D(ctypes.Structure):
    """``bella_adv3d``: device arrays of the 3D advection (reference layout)."""
    _fields_ = [("inx", ctypes.c_int), ("iny", ctypes.c_int), ("inz", ctypes.c_int),
                ("x_wall", ctypes.c_int), ("y_wall", ctypes.c_int), ("z_wall", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("g", ctypes.c_double), ("gamm", ctypes.c_double),
                ("is_compressible", ctypes.c_int), ("pad_", ctypes.c_int)] + \
        [(k, _dp) for k in ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")] + \
        [("fx", _dp * 6), ("fy", _dp * 6), ("fz", _dp * 6), ("hydro_rhoY0", _dp), ("strat_inv", _dp),
         ("pwchi", _dp)]


class Expl3D(ctypes.Structure):
    """``bella_expl3d``: device arrays of the 3D explicit projection parts."""
    _fields_ = [("inx", ctypes.c_int), ("iny", ctypes.c_int), ("inz", ctypes.c_int),
                ("x_wall", ctypes.c_int), ("y_wall", ctypes.c_int), ("z_wall", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
                ("Msq", ctypes.c_double), ("g", ctypes.c_double), ("gamm", ctypes.c_double),
                ("nonhydro", ctypes.c_double), ("compressibility", ctypes.c_double),
                ("coriolis", ctypes.c_double * 3), ("wind", ctypes.c_double * 3),
                ("is_compressible", ctypes.c_int), ("is_ArakawaKonor", ctypes.c_int)] + \
        [(k, _dp) for k in ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX", "p2", "rhs_out", "scratch",
                            "S0c", "S0n", "hydro_rhoY0", "strat_inv")] + \
        [("div_sign_2d", ctypes.c_int)]


class Expl2D(ctypes.Structure):
    _fields_ = [("inx", ctypes.c_int), ("iny", ctypes.c_int), ("x_wall", ctypes.c_int), ("y_wall", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dt", ctypes.c_double),
                ("Msq", ctypes.c_double), ("g", ctypes.c_double), ("gamm", ctypes.c_double),
                ("nonhydro", ctypes.c_double), ("compressibility", ctypes.c_double),
                ("coriolis", ctypes.c_double * 3), ("wind", ctypes.c_double * 3),
                ("is_compressible", ctypes.c_int), ("is_ArakawaKonor", ctypes.c_int)] + \
        [(k, ctypes.c_void_p) for k in ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX", "p2", "rhs_out",
                                         "S0c", "S0n", "hydro_rhoY0", "strat_inv")]


class SolveOpts(ctypes.Structure):
    """``bella_solve_opts``."""
    _fields_ = [("tol", ctypes.c_double), ("atol", ctypes.c_double),
                ("maxiter", ctypes.c_int), ("precision", ctypes.c_int),
                ("x0_zero", ctypes.c_int), ("project_null", ctypes.c_int),
                ("inner_tol", ctypes.c_double), ("max_outer", ctypes.c_int),
                ("check_every", ctypes.c_int), ("timeout_s", ctypes.c_double)]


class SolveStats(ctypes.Structure):
    """``bella_solve_stats``."""
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int),
                ("outer", ctypes.c_int), ("matvecs", ctypes.c_int),
                ("relres", ctypes.c_double), ("bnorm", ctypes.c_double),
                ("seconds", ctypes.c_double), ("fallback", ctypes.c_int), ("detail", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# exported symbol -> (restype, argtypes); also the list checked by the tests
SIGNATURES = {
    "bella_ws_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]),
    "bella_ws_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "bella_last_error": (ctypes.c_char_p, []),
    "bella_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "bella_version": (ctypes.c_int, []),
    "bella_ws_launches": (ctypes.c_longlong, [ctypes.c_void_p]),
    "bella_ws_profile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "bella_ws_kernel_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_longlong)]),
    "bella_op2d_set": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Op2D), ctypes.c_void_p]),
    "bella_op3d_set": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Op3D), ctypes.c_void_p]),
    "bella_apply_f64": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, ctypes.c_void_p]),
    "bella_apply_f32": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, ctypes.c_void_p]),
    "bella_solve_opts_default": (None, [ctypes.POINTER(SolveOpts)]),
    "bella_bicgstab": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, ctypes.POINTER(SolveOpts),
                                      ctypes.POINTER(SolveStats), ctypes.c_void_p]),
    "bella_projection2d": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Proj2D), ctypes.POINTER(SolveOpts),
                                          ctypes.POINTER(SolveStats), ctypes.c_void_p]),
    "bella_projection2d_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                  ctypes.POINTER(SolveOpts), ctypes.c_int, ctypes.c_void_p,
                                                  ctypes.c_void_p]),
    "bella_projection3d": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Proj3D), ctypes.POINTER(SolveOpts),
                                          ctypes.POINTER(SolveStats), ctypes.c_void_p]),
    "bella_advective_fluxes2d": (ctypes.c_int, [ctypes.POINTER(Adv2D), ctypes.c_void_p]),
    "bella_advect2d": (ctypes.c_int, [ctypes.POINTER(Adv2D), ctypes.c_double, ctypes.c_int, ctypes.c_void_p]),
    "bella_advect_rk2d": (ctypes.c_int, [ctypes.POINTER(Adv2D), ctypes.c_double, ctypes.c_void_p]),
    "bella_boundary2d": (ctypes.c_int, [ctypes.POINTER(Adv2D), ctypes.c_void_p]),
    "bella_advective_fluxes3d": (ctypes.c_int, [ctypes.POINTER(Adv3D), ctypes.c_void_p]),
    "bella_advect3d": (ctypes.c_int, [ctypes.POINTER(Adv3D), ctypes.c_double, ctypes.c_int, ctypes.c_void_p]),
    "bella_advect_rk3d": (ctypes.c_int, [ctypes.POINTER(Adv3D), ctypes.c_double, ctypes.c_void_p]),
    "bella_boundary3d": (ctypes.c_int, [ctypes.POINTER(Adv3D), ctypes.c_void_p]),
    "bella_euler_forward3d": (ctypes.c_int, [ctypes.POINTER(Expl3D), ctypes.c_void_p]),
    "bella_cfl_maxima": (ctypes.c_int, [ctypes.c_void_p] * 5 + [ctypes.c_longlong, ctypes.c_double, ctypes.c_double,
                                                                  ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                                                  ctypes.c_void_p]),
    "bella_expl_part3d": (ctypes.c_int, [ctypes.POINTER(Expl3D), ctypes.c_void_p]),
    "bella_cnn_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int,
                                        ctypes.c_longlong]),
    "bella_cnn_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "bella_cnn_param_count": (ctypes.c_longlong, [ctypes.c_int]),
    "bella_cnn_block": (ctypes.c_int, [ctypes.c_void_p]),
    "bella_cnn_set_mode": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "bella_cnn_set_skip": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float]),
    "bella_cnn_set_tc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "bella_cnn_tc_error": (ctypes.c_int, [ctypes.c_void_p]),
    "bella_cnn_train_step_op": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                               ctypes.c_float,
                                               ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
    "bella_crop_apply": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, _dp, _dp, ctypes.c_void_p]),
    "bella_bicgstab_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.POINTER(SolveOpts), ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p]),
    "bella_batch_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
    "bella_batch_config_count": (ctypes.c_int, []),
    "bella_batch_config": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_int)]),
    "bella_euler_forward2d": (ctypes.c_int, [ctypes.POINTER(Expl2D), ctypes.c_void_p]),
    "bella_expl_part2d": (ctypes.c_int, [ctypes.POINTER(Expl2D), ctypes.c_void_p]),
    "bella_fbicgstab": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, _dp, _dp, ctypes.POINTER(SolveOpts),
                                       ctypes.POINTER(SolveStats), ctypes.c_void_p]),
    "bella_spectral3d_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Op3D), ctypes.c_int,
                                               ctypes.c_void_p]),
    "bella_spectral2d_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Op2D), ctypes.c_int,
                                               ctypes.c_void_p]),
    "bella_spectral3d_update": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Op3D), ctypes.c_void_p]),
    "bella_spectral2d_update": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Op2D), ctypes.c_void_p]),
    "bella_spectral3d_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "bella_spectral3d_apply": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, ctypes.c_void_p]),
    "bella_spectral3d_launches": (ctypes.c_longlong, [ctypes.c_void_p]),
    "bella_fbicgstab_pc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _dp, _dp,
                                          ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), ctypes.c_void_p]),
    "bella_fgmres_pc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                       _dp, _dp, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats),
                                       ctypes.c_void_p]),
    "bella_cnn_set_params": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_void_p]),
    "bella_cnn_get_params": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_void_p]),
    "bella_cnn_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                         ctypes.c_float, ctypes.c_void_p]),
    "bella_cnn_gradients": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp,
                                           _dp, ctypes.c_void_p]),
    "bella_cnn_train_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            _dp, _dp, ctypes.c_float, ctypes.POINTER(ctypes.c_double),
                                            ctypes.c_void_p]),
    "bella_cnn_launches": (ctypes.c_longlong, [ctypes.c_void_p]),
    "bella_bicgstab2d_noalloc": (ctypes.c_int, [ctypes.POINTER(Op2D), _dp, _dp, ctypes.POINTER(SolveOpts),
                                                ctypes.POINTER(SolveStats), ctypes.c_void_p]),
}

_lib = None


def load():
    """Load the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "libbella_gb300.so is not built (%s); run `python -m pybella_gb300.build` "
            "(needs nvcc).  There is no CPU fallback." % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class BellaError(RuntimeError):
    pass


def check(rc, what):
    """Raise :class:`BellaError` for a negative (error) return code."""
    if rc < 0:
        lib = load()
        raise BellaError("%s failed (%d: %s): %s" % (
            what, rc, lib.bella_status_string(rc).decode(), lib.bella_last_error().decode()))
    return rc


class Workspace:
    """Owns one ``bella_ws`` handle on a CUDA device."""

    def __init__(self, device=0):
        self._lib = load()
        h = ctypes.c_void_p()
        check(self._lib.bella_ws_create(ctypes.byref(h), int(device)), "bella_ws_create")
        self.handle = h
        self.device = int(device)

    @property
    def launches(self):
        return int(self._lib.bella_ws_launches(self.handle))

    def profile(self, enable=True):
        check(self._lib.bella_ws_profile(self.handle, int(bool(enable))), "bella_ws_profile")

    def kernel_time(self, kind):
        """(total ms, launches) of one solver kernel kind since profiling was enabled."""
        t = ctypes.c_double()
        c = ctypes.c_longlong()
        check(self._lib.bella_ws_kernel_time(self.handle, int(kind), ctypes.byref(t), ctypes.byref(c)),
              "bella_ws_kernel_time")
        return t.value, c.value

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self._lib.bella_ws_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
