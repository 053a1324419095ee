"""ctypes binding of libandromeda_gb300.so (the C ABI in include/andromeda_gb300.h).

The shared library is built in-tree by :mod:`andromeda_gb300.build`.  There is
no fallback: if the library is missing or cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libandromeda_gb300.so")

# Every symbol the header declares, with its ctypes signature.
dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
vp = C.c_void_p
I = C.c_int
D = C.c_double
PI = C.POINTER(C.c_int)

SIGNATURES = {
    "agb_version": ([], C.c_char_p),
    "agb_create": ([C.POINTER(vp), I], I),
    "agb_destroy": ([vp], I),
    "agb_last_error": ([vp], C.c_char_p),
    "agb_set_mesh": ([vp, I, dp, I, ip, ip, ip], I),
    "agb_set_problem": ([vp, I, I, ip, dp, D, ip, I, I], I),
    "agb_get_geometry": ([vp, dp, dp, dp], I),
    "agb_set_integration": ([vp, I, I, D, I], I),
    "agb_set_node_walls": ([vp, I, vp], I),
    "agb_set_solver": ([vp, I], I),
    "agb_set_gmres_restart": ([vp, I], I),
    "agb_set_residual_mode": ([vp, I], I),
    "agb_surface_pressure": ([vp, dp, dp, dp], I),
    "agb_domain_values": ([vp, I, dp, dp, dp, dp, dp], I),
    "agb_system_size": ([vp, PI, PI], I),
    "agb_assemble": ([vp, I], I),
    "agb_get_system": ([vp, I, vp, vp], I),
    "agb_rhs": ([vp, I, dp, dp], I),
    "agb_solve": ([vp, I, dp, dp, I, D, I, ip, ip], I),
    "agb_force_torque": ([vp, I, dp, I, dp], I),
    "agb_resistance_tensor": ([vp, I, I, I, I, D, I, dp, ip, ip, dp], I),
    "agb_kernel_times": ([vp, I, dp], I),
    "agb_lsqr_precon": ([I, I, C.c_int64, dp, lp, ip, dp], I),
    "agb_lsqr_solve": ([I, I, C.c_int64, PI, D, PI, PI, dp, lp, ip, dp, dp, dp], I),
    "agb_lsqr_precon_dense_noalloc": ([I, I, C.c_int64, vp, vp], I),
    "agb_selftest_bounded_wait": ([I, C.c_uint, I, C.POINTER(C.c_int)], I),
    "agb_mesh_read": ([C.c_char_p, ip, vp, vp, vp, vp, vp, C.c_char_p, I], I),
    "agb_vtu_write": ([C.c_char_p, I, I, dp, I, ip, ip, ip, dp, I, C.POINTER(C.c_char_p), dp, dp, vp], I),
    "agb_integrals_file_write": ([C.c_char_p, I, I, I, I, dp, dp, dp], I),
    "agb_integrals_file_read": ([C.c_char_p, I, ip, dp, vp, vp], I),
    "agb_integral_matrices": ([vp, vp, vp, vp], I),
    "agb_layout_sizes": ([vp, ip], I),
    "agb_solve_fields": ([vp, I, dp, vp, dp, dp, I, D, I, ip, ip], I),
    "agb_form_pre_fm": ([I, I, dp, dp, C.POINTER(C.c_float), PI], I),
    "agb_solv_eqn_fm": ([I, I, I, I, I, D, I, dp, dp, dp, dp, PI, C.POINTER(C.c_double), PI], I),
    "agb_solve_lu": ([vp, I, dp, dp, PI], I),
    "agb_mlp_create": ([C.POINTER(vp), I, I, I, I, C.c_ulonglong], I),
    "agb_mlp_destroy": ([vp], I),
    "agb_mlp_num_params": ([vp, C.POINTER(C.c_longlong)], I),
    "agb_mlp_get_params": ([vp, fp], I),
    "agb_mlp_set_params": ([vp, fp], I),
    "agb_mlp_set_normalization": ([vp, fp, fp, fp, fp], I),
    "agb_mlp_gradient": ([vp, I, fp, fp, I, fp, C.POINTER(C.c_double)], I),
    "agb_mlp_train": ([vp, I, fp, fp, I, I, C.c_float, C.c_ulonglong, dp, dp], I),
    "agb_mlp_predict": ([vp, I, fp, fp, I, C.POINTER(C.c_double)], I),
    "agb_mlp_launches": ([vp], C.c_longlong),
    "agb_batch_resistance": ([vp, I, ip, dp, ip, ip, ip, ip, I, I, I, I, D, D, I, dp, ip, ip, dp], I),
}

_lib = None


class AgbError(RuntimeError):
    pass


def load(path: str | None = None):
    """Load the CUDA library (raises if it is absent: no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise AgbError(f"{p} is missing: build it with `python -m andromeda_gb300.build` "
                       "(the GPU path has no fallback)")
    L = C.CDLL(p)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L
