"""ctypes binding of the C ABI declared in include/cosmos_gb300.h.

The library is built in-tree (cosmos_gb300/libcosmos_gb300.so, see cosmos_gb300/build.py).
Loading fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcosmos_gb300.so")

OK, EINVAL, ECUDA, ENONFINITE, EUNSUPPORTED, ESTATE = 0, 1, 2, 3, 4, 5
STATUS_NONFINITE, STATUS_NEWTON_CAP = 1, 2
NEWTONIAN, SR, GR = 0, 1, 2
FP64, FP32 = 0, 1
BC_TRANSMISSIVE, BC_PERIODIC = 0, 1
SUPERBEE, VANLEER, MINBEE = 0, 1, 2
(STATE_CONS, STATE_PRIM, STATE_FLUX_X, STATE_FLUX_Y, STATE_SOUND, STATE_INTERNAL_ENERGY, STATE_TOTAL_ENERGY,
 STATE_PRESSURE, STATE_ENTHALPY, STATE_SOURCE, STATE_EIGENVALUES, STATE_GRADIENT_RATIO, STATE_LIMITER,
 STATE_SLOPE) = range(14)
# every public quantity of BlackHoleSpacetime at a point (cosmos_spacetime_eval, COSMOS_ST_* offsets)
SPACETIME_WIDTH = 125
# per-interface solver functions (cosmos_interface_eval), the public COSMOS_IF_* codes
(IF_LAX_FRIEDRICHS, IF_RICHTMYER, IF_FORCE, IF_FORCE_UPDATE, IF_FRACTIONAL_EVOLUTION, IF_EVOLUTION,
 IF_X_LAX_FRIEDRICHS_FLUX, IF_Y_LAX_FRIEDRICHS_FLUX, IF_X_RICHTMYER_FLUX, IF_Y_RICHTMYER_FLUX, IF_X_FORCE_FLUX,
 IF_Y_FORCE_FLUX, IF_X_SLIC_FLUX, IF_Y_SLIC_FLUX, IF_EVOLVE_HALF_X, IF_EVOLVE_HALF_Y, IF_EVOLVE_HALF_VECTOR_X,
 IF_EVOLVE_HALF_VECTOR_Y, IF_EVOLVE_FRACTION_X, IF_EVOLVE_FRACTION_Y, IF_EVOLVE_FRACTION_VECTOR, IF_RK_CELL_1D,
 IF_RK_CELL_2D) = range(23)


class Params(ctypes.Structure):
    _fields_ = [("system", ctypes.c_int), ("dims", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("precision", ctypes.c_int), ("boundary", ctypes.c_int), ("gamma", ctypes.c_double),
                ("dx", ctypes.c_double), ("bh_mass", ctypes.c_double), ("bh_spin", ctypes.c_double),
                ("bh_x", ctypes.c_double), ("bh_y", ctypes.c_double), ("bh_z", ctypes.c_double),
                ("sr_c2p64_above", ctypes.c_double)]


class AmrResult(ctypes.Structure):
    _fields_ = [("coarse_steps", ctypes.c_int), ("fine_steps", ctypes.c_int), ("t", ctypes.c_double),
                ("status", ctypes.c_int), ("fine_run", ctypes.c_int), ("mid_run", ctypes.c_int)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("cfl", ctypes.c_double), ("t_final", ctypes.c_double),
                ("bias", ctypes.c_double), ("limiter", ctypes.c_int), ("subcycles", ctypes.c_int),
                ("max_steps", ctypes.c_int)]


class SolveResult(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("t", ctypes.c_double), ("status", ctypes.c_int)]


# exported symbol -> (restype, argtypes); the single source of truth for the binding and for
# the CPU test that checks the library exports every function the header declares
_p, _i, _d, _sz, _u8p = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t, ctypes.c_void_p
SIGNATURES = {
    "cosmos_version": (ctypes.c_char_p, []),
    "cosmos_last_error": (ctypes.c_char_p, []),
    "cosmos_kernel_launches": (ctypes.c_ulonglong, []),
    "cosmos_set_tensor_maps": (_i, [_i]),
    "cosmos_params_default": (None, [ctypes.POINTER(Params)]),
    "cosmos_solve_opts_default": (None, [ctypes.POINTER(SolveOpts)]),
    "cosmos_stable_dt_rule": (_d, [_d, _d, _d, _i]),
    "cosmos_ctx_create": (_i, [_i, ctypes.POINTER(_p)]),
    "cosmos_ctx_destroy": (_i, [_p]),
    "cosmos_ctx_synchronize": (_i, [_p]),
    "cosmos_ctx_stream": (_p, [_p]),
    "cosmos_grid_create": (_i, [_p, ctypes.POINTER(Params), ctypes.POINTER(_p)]),
    "cosmos_grid_destroy": (_i, [_p]),
    "cosmos_grid_set_prim": (_i, [_p, _p, _sz]),
    "cosmos_grid_get_prim": (_i, [_p, _p, _sz]),
    "cosmos_grid_sweep": (_i, [_p, _i, _i, _d, _d, _i]),
    "cosmos_grid_rk_source": (_i, [_p, _d, _d, _i]),
    "cosmos_grid_max_wavespeed": (_i, [_p, ctypes.POINTER(_d)]),
    "cosmos_grid_stable_dt": (_i, [_p, _d, _d, _d, _i, ctypes.POINTER(_d)]),
    "cosmos_grid_solve": (_i, [_p, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveResult)]),
    "cosmos_grid_run_begin": (_i, [_p, ctypes.POINTER(SolveOpts)]),
    "cosmos_grid_run_steps": (_i, [_p, _i]),
    "cosmos_grid_run_end": (_i, [_p, ctypes.POINTER(SolveResult)]),
    "cosmos_grid_field_sums": (_i, [_p, _p]),
    "cosmos_grid_amr_flags": (_i, [_p, _d, _u8p, _u8p]),
    "cosmos_grid_amr_derefine": (_i, [_p, _p, _d, _u8p, _u8p]),
    "cosmos_solve_prim": (_i, [ctypes.POINTER(Params), _p, _p, ctypes.POINTER(SolveOpts),
                               ctypes.POINTER(SolveResult)]),
    "cosmos_field_sums_noalloc": (_i, [_p, _i, _i, _i, _i, _sz, _p, _p]),
    "cosmos_grid_adjoint": (_i, [_p, ctypes.POINTER(SolveOpts), _i, _i, _p, _p, _p, _p, _p, _p]),
    "cosmos_grid_set_adjoint_keep": (_i, [_p, ctypes.c_longlong]),
    "cosmos_amr_create": (_i, [_p, ctypes.POINTER(Params), ctypes.POINTER(_p)]),
    "cosmos_amr_create_level2": (_i, [_p, ctypes.POINTER(Params), ctypes.POINTER(_p)]),
    "cosmos_amr_get_level": (_i, [_p, _i, _p, _p]),
    "cosmos_amr_destroy": (_i, [_p]),
    "cosmos_amr_set_prim": (_i, [_p, _p, _sz]),
    "cosmos_amr_solve": (_i, [_p, _d, _d, _d, _i, ctypes.POINTER(AmrResult)]),
    "cosmos_amr_get": (_i, [_p, _p, _p, _p, _p]),
    "cosmos_state_width": (_i, [_i, ctypes.POINTER(_sz), ctypes.POINTER(_sz)]),
    "cosmos_state_eval": (_i, [_p, ctypes.POINTER(Params), _i, _sz, _p, _p, _d, _i, _p]),
    "cosmos_batch_create": (_i, [_p, _i, _p, _p, _p, _p, _d, _i, _i, ctypes.POINTER(_p)]),
    "cosmos_batch_destroy": (_i, [_p]),
    "cosmos_batch_size": (_i, [_p, ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_longlong)]),
    "cosmos_batch_set_prim": (_i, [_p, _i, _p, _sz]),
    "cosmos_batch_get_prim": (_i, [_p, _i, _p, _sz]),
    "cosmos_batch_run_begin": (_i, [_p, ctypes.POINTER(SolveOpts)]),
    "cosmos_batch_run_steps": (_i, [_p, _i]),
    "cosmos_batch_run_end": (_i, [_p, _p]),
    "cosmos_batch_set_shape": (_i, [_p, _i, _i, _i]),
    "cosmos_batch_set_wait_limit": (_i, [_p, ctypes.c_longlong]),
    "cosmos_interface_width": (_i, [_i, ctypes.POINTER(_sz), ctypes.POINTER(_sz)]),
    "cosmos_spacetime_eval": (_i, [_p, ctypes.POINTER(Params), _sz, _p, _p]),
    "cosmos_interface_eval": (_i, [_p, ctypes.POINTER(Params), _i, _sz, _p, _p, _d, _d, _i, _d, _i, _p]),
    "cosmos_batch_time_shape": (_i, [_p, _i, _i, _i, _i, ctypes.POINTER(_d)]),
    "cosmos_batch_autotune": (_i, [_p, ctypes.c_char_p, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i),
                                   ctypes.POINTER(_d)]),
}

_lib = None


class CosmosError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cosmos error {code}: {msg}")
        self.code = code


def load(path=LIB_PATH):
    """Load the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m cosmos_gb300.build` "
                           "(this package has no CPU fallback)")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != OK:
        msg = load().cosmos_last_error()
        raise CosmosError(rc, msg.decode() if msg else "")
    return rc
