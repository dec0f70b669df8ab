"""ctypes binding of libilm.so (the C ABI declared in include/ilm.h).

The library is built in-tree by ``immersedlayers._build.build()``.  Loading
fails loudly if it is missing: there is no CPU fallback for any operator.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libilm.so")

# enums (include/ilm.h)
ILM_OK = 0
ILM_ERR_NOT_CONVERGED = 4
F64, F32 = 0, 1
DDF = {"Yang3": 0, "Roma": 1, "M4prime": 2, "Witchhat": 3, "M3": 4}
GRID_SCALING, INDEX_SCALING = 0, 1
STOKES_MAX_RHS = 32
CACHE_SCALAR, CACHE_VECTOR = 0, 1
NODES_PRIMAL, NODES_DUAL, EDGES_PRIMAL, EDGES_DUAL, EDGEGRAD_PRIMAL = 0, 1, 2, 3, 4
SCALAR_DATA, VECTOR_DATA, TENSOR_DATA = 0, 1, 2
SCHUR = {"RTLinvR": 0, "CLinvCT": 1, "GLinvD": 2, "nRTRn": 3, "CLinvCT_scalar": 4, "CL2invCT": 5, "GLinvD_symm": 6,
         "GLinvD_cross": 7}


class ILMError(RuntimeError):
    """Raised when a libilm call returns a non-zero status."""

    def __init__(self, status, func, msg):
        super().__init__(f"{func} failed with status {status}: {msg}")
        self.status = status


class BatchProblem(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("h", C.c_double), ("i0x", C.c_int), ("i0y", C.c_int),
                ("npts", C.c_int), ("kind", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("rel_residual", C.c_double)]


_VP = C.c_void_p
_I = C.c_int
_D = C.c_double
_DP = C.POINTER(C.c_double)

# name -> argtypes (all return int unless listed in _RESTYPES)
SIGNATURES = {
    "ilm_version": [],
    "ilm_status_string": [_I],
    "ilm_last_error": [],
    "ilm_grid_create": [_I, _I, _D, _I, _I, C.POINTER(_VP)],
    "ilm_grid_destroy": [_VP],
    "ilm_grid_numel": [_VP, _I, C.POINTER(C.c_size_t)],
    "ilm_alloc": [C.c_size_t, C.POINTER(_VP)],
    "ilm_free": [_VP],
    "ilm_copy_h2d": [_VP, _VP, C.c_size_t, _VP],
    "ilm_copy_d2h": [_VP, _VP, C.c_size_t, _VP],
    "ilm_cache_create": [_VP, _I, _I, _DP, _DP, _DP, _DP, _DP, _I, _I, _I, C.POINTER(_VP)],
    "ilm_cache_destroy": [_VP],
    "ilm_cache_update_points": [_VP, _VP, _VP, _VP, _VP, _VP, _VP],
    "ilm_cache_npts": [_VP, C.POINTER(_I)],
    "ilm_regularize": [_VP, _I, _VP, _VP, _VP],
    "ilm_regularize_add": [_VP, _I, _VP, _VP, _VP],
    "ilm_grid_mul_add": [C.c_size_t, _I, _VP, _VP, _VP, _VP],
    "ilm_interpolate": [_VP, _I, _VP, _VP, _VP],
    "ilm_surface_filter": [_VP, _I, _VP, _VP, _VP],
    "ilm_regularize_normal": [_VP, _VP, _VP, _VP],
    "ilm_regularize_normal_symm": [_VP, _VP, _VP, _VP],
    "ilm_regularize_normal_cross": [_VP, _I, _VP, _VP, _VP],
    "ilm_regularize_normal_dot": [_VP, _I, _VP, _VP, _VP],
    "ilm_normal_interpolate": [_VP, _VP, _VP, _VP],
    "ilm_normal_interpolate_symm": [_VP, _VP, _VP, _VP],
    "ilm_normal_cross_interpolate": [_VP, _I, _VP, _VP, _VP],
    "ilm_normal_dot_interpolate": [_VP, _I, _VP, _VP, _VP],
    "ilm_surface_divergence": [_VP, _VP, _VP, _VP],
    "ilm_surface_divergence_symm": [_VP, _VP, _VP, _VP],
    "ilm_surface_grad": [_VP, _VP, _VP, _VP],
    "ilm_surface_grad_symm": [_VP, _VP, _VP, _VP],
    "ilm_surface_curl": [_VP, _I, _I, _VP, _VP, _VP],
    "ilm_surface_curl_cross": [_VP, _I, _VP, _VP, _VP],
    "ilm_surface_divergence_cross": [_VP, _VP, _VP, _VP],
    "ilm_surface_grad_cross": [_VP, _VP, _VP, _VP],
    "ilm_divergence": [_VP, _I, _VP, _VP, _VP],
    "ilm_grad": [_VP, _I, _VP, _VP, _VP],
    "ilm_curl": [_VP, _I, _VP, _VP, _VP],
    "ilm_laplacian": [_VP, _I, _VP, _VP, _VP],
    "ilm_convective_derivative": [_VP, _I, _VP, _VP, _VP, _VP],
    "ilm_w_cross_v": [_VP, _VP, _VP, _VP, _VP],
    "ilm_vecfield_helmholtz": [_VP, _VP, _VP, _VP, _VP, _DP, _VP, _VP],
    "ilm_inverse_laplacian": [_VP, _I, _VP, _VP, _VP],
    "ilm_mask": [_VP, _I, _I, _VP, _VP],
    "ilm_dot_grid": [_VP, _I, _VP, _VP, _DP, _VP],
    "ilm_dot_surface": [_VP, _I, _VP, _VP, _DP, _VP],
    "ilm_dot_grid_noalloc": [_I, _I, _D, _I, _I, _I, _VP, _VP, _DP, _VP],
    "ilm_schur_build": [_VP, _I, _D, _VP, _VP],
    "ilm_solve_dirichlet": [_VP, _VP, _VP, _VP, _VP, _D, _I, C.POINTER(SolveInfo), _VP],
    "ilm_solve_neumann": [_VP, _VP, _VP, _VP, _VP, _D, _I, C.POINTER(SolveInfo), _VP],
    "ilm_solve_dirichlet_refined": [_VP, _VP, _VP, _VP, _VP, _D, _I, _I, C.POINTER(SolveInfo), _VP],
    "ilm_solve_neumann_refined": [_VP, _VP, _VP, _VP, _VP, _D, _I, _I, C.POINTER(SolveInfo), _VP],
    "ilm_solve_neumann_full": [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _D, _I, C.POINTER(SolveInfo), _VP],
    "ilm_solve_stokes": [_VP, _VP, _VP, _VP, _VP, _VP, _D, _I, C.POINTER(SolveInfo), _VP],
    "ilm_solve_stokes_multi": [_VP, _I, _VP, _VP, _VP, _VP, _VP, _D, _I, _I, C.POINTER(SolveInfo), _VP],
    "ilm_solve_stokes_multi_refined": [_VP, _I, _VP, _VP, _VP, _VP, _VP, _D, _I, _I, C.POINTER(SolveInfo), _VP],
    "ilm_batch_create": [_I, C.POINTER(BatchProblem), _DP, _DP, _DP, _DP, _DP, _I, _I, C.POINTER(_VP)],
    "ilm_batch_destroy": [_VP],
    "ilm_batch_layout": [_VP, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)],
    "ilm_batch_solve": [_VP, _VP, _VP, _VP, _VP, _D, _I, _VP],
    "ilm_batch_solve_graph": [_VP, _VP, _VP, _VP, _VP, _D, _I, _VP],
    "ilm_batch_solve_refined": [_VP, _VP, _VP, _VP, _VP, _D, _I, _I, _VP],
    "ilm_batch_info": [_VP, C.POINTER(_I), _DP],
    "ilm_batch_set_precond": [_VP, _I, _I],
    "ilm_batch_set_profiling": [_VP, _I],
    "ilm_batch_stage_times": [_VP, C.POINTER(C.c_float), C.POINTER(_I), C.POINTER(_I)],
    "ilm_batch_cg_times": [_VP, _DP, _DP, C.POINTER(_I)],
    "ilm_batch_set_cg_variant": [_VP, _I],
    "ilm_batch_set_rhs_operator": [_VP, _I],
    "ilm_batch_get_cg_variant": [_VP, C.POINTER(_I), C.POINTER(_I)],
    "ilm_batch_autotune": [_VP, _VP, _VP, _VP, _VP, C.c_double, _I, _I, _VP, C.POINTER(_I), C.POINTER(C.c_float)],
    "ilm_batch_stats": [_VP, _DP],
    "ilm_batch_setup_times": [_VP, _DP, _I, C.POINTER(_I), C.POINTER(C.c_char_p)],
    "ilm_net_create": [_I, _I, _I, _I, C.POINTER(_VP)],
    "ilm_net_destroy": [_VP],
    "ilm_net_set_tensor_cores": [_VP, _I],
    "ilm_net_nparams": [_VP, C.POINTER(C.c_size_t)],
    "ilm_net_set_params": [_VP, C.POINTER(C.c_float)],
    "ilm_net_get_params": [_VP, C.POINTER(C.c_float)],
    "ilm_net_forward": [_VP, _I, _VP, _VP, _VP, _VP, _VP],
    "ilm_net_loss_grad": [_VP, _I, _I, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _DP, C.POINTER(C.c_float), _VP],
    "ilm_net_train_step": [_VP, _I, _I, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _D, _VP, _VP],
    "ilm_point_features": [_I, _DP, _DP, _DP, _DP, _DP, C.POINTER(_I), C.POINTER(_I), _D, C.POINTER(C.c_float)],
    "ilm_batch_set_learned": [_VP, _VP, _I, C.POINTER(_I)],
    "ilm_batch_set_coarse": [_VP, _I, C.POINTER(C.c_int)],
    "ilm_batch_schur_apply": [_VP, _VP, _VP, _VP],
    "ilm_batch_schur_solve": [_VP, _VP, _VP, _D, _I, _VP],
    "ilm_heat_create": [_VP, _D, _D, _DP, _DP, _D, _I, C.POINTER(_VP)],
    "ilm_heat_destroy": [_VP],
    "ilm_heat_advance": [_VP, _VP, _VP, _I, _VP],
    "ilm_heat_info": [_VP, C.POINTER(_I), _DP, C.POINTER(C.c_size_t)],
}
_RESTYPES = {"ilm_status_string": C.c_char_p, "ilm_last_error": C.c_char_p}

# functions that may legitimately return ILM_ERR_NOT_CONVERGED (reported via info)
_SOFT = {"ilm_solve_dirichlet", "ilm_solve_neumann", "ilm_solve_neumann_full", "ilm_solve_stokes",
         "ilm_solve_stokes_multi", "ilm_solve_stokes_multi_refined",
         "ilm_solve_dirichlet_refined", "ilm_solve_neumann_refined"}

_lib = None
_lock = threading.Lock()


def exported_symbols():
    """Names the header declares (the ABI this binding expects)."""
    return sorted(SIGNATURES)


def load(path: str | None = None):
    """Load libilm.so (raises OSError when it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise OSError(f"libilm.so not found at {p}; build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(p)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, C.c_int)
        _lib = lib
        return lib


def call(name, *args):
    """Call a libilm function and raise ILMError on a non-zero status."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != ILM_OK and not (st == ILM_ERR_NOT_CONVERGED and name in _SOFT):
        msg = lib.ilm_last_error().decode(errors="replace")
        raise ILMError(st, name, msg)
    return st
