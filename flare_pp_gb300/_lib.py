"""ctypes binding of libflare_pp_gb300.so (the C ABI in include/flare_pp_gb300.h).

The library is built in-tree by ``flare_pp_gb300.build``.  Loading fails with
an error when it is missing: there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libflare_pp_gb300.so")

FPP_OK = 0
FPP_ERR_INVALID = -1
FPP_ERR_CUDA = -2
FPP_ERR_OOM = -3
FPP_ERR_TIMEOUT = -4
FPP_ERR_UNSUPPORTED = -5
FPP_ERR_CAPACITY = -6
FPP_ERR_NUMERIC = -7
FPP_PREC_FP64 = 0
FPP_PREC_MIXED = 1

_c_int = ctypes.c_int
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_dbl = ctypes.c_double
_vp = ctypes.c_void_p
_cp = ctypes.c_char_p
_P = ctypes.POINTER

# name -> (restype, argtypes); mirrors include/flare_pp_gb300.h
SIGNATURES = {
    "fpp_last_error": (_cp, []),
    "fpp_version": (_c_int, []),
    "fpp_structure_create": (_c_int, [_vp, _vp, _vp, _i32, _dbl, _vp, _P(_vp)]),
    "fpp_structure_set_positions": (_c_int, [_vp, _vp, _c_int, _vp]),
    "fpp_structure_destroy": (_c_int, [_vp]),
    "fpp_structure_info": (_c_int, [_vp, _P(_i32), _P(_i64), _P(_i32), _P(_dbl)]),
    "fpp_structure_get_neighbors": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fpp_structure_set_profiling": (_c_int, [_vp, _c_int]),
    "fpp_structure_stage_times": (_c_int, [_vp, _vp]),
    "fpp_b2_create": (_c_int, [_cp, _cp, _vp, _i32, _vp, _i32, _vp, _vp, _P(_vp)]),
    "fpp_b3_create": (_c_int, [_cp, _cp, _vp, _i32, _vp, _i32, _vp, _P(_vp)]),
    "fpp_b2_destroy": (_c_int, [_vp]),
    "fpp_b2_n_descriptors": (_c_int, [_vp, _P(_i32)]),
    "fpp_b2_pair_count": (_c_int, [_vp, _vp, _P(_i64), _vp]),
    "fpp_b2_compute": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fpp_b2_descriptors_noalloc": (_c_int, [_vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fpp_structure_set_skin": (_c_int, [_vp, _dbl, _vp]),
    "fpp_structure_neighbor_stats": (_c_int, [_vp, _P(_i64), _P(_i64), _P(_dbl)]),
    "fpp_predict_mapped_batched": (_c_int, [_vp, _vp, _i32, _c_int, _vp, _vp, _vp, _vp]),
    "fpp_dgemm_nt": (_c_int, [_i32, _i32, _i32, _vp, _i64, _vp, _i64, _vp, _i64, _i32, _vp]),
    "fpp_model_create": (_c_int, [_vp, _dbl, _dbl, _P(_vp)]),
    "fpp_model_destroy": (_c_int, [_vp]),
    "fpp_model_set_sparse": (_c_int, [_vp, _i32, _i32, _vp, _vp, _vp]),
    "fpp_model_set_R_inv": (_c_int, [_vp, _i32, _vp]),
    "fpp_model_compute_beta": (_c_int, [_vp, _vp, _vp]),
    "fpp_model_set_beta": (_c_int, [_vp, _i32, _vp]),
    "fpp_envs_envs": (_c_int, [_vp, _vp, _vp, _vp]),
    "fpp_envs_struc": (_c_int, [_vp, _vp, _vp, _vp]),
    "fpp_local_uncertainties": (_c_int, [_vp, _vp, _vp, _i32, _vp, _vp]),
    "fpp_predict_energy_uncertainty": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fpp_kuf_batched": (_c_int, [_vp, _vp, _i32, _vp, _vp, _vp, _vp, _i64, _vp]),
    "fpp_struc_struc": (_c_int, [_vp, _dbl, _dbl, _vp, _vp, _vp, _vp]),
    "fpp_self_kernel_struc": (_c_int, [_vp, _dbl, _dbl, _vp, _vp, _vp]),
    "fpp_predict": (_c_int, [_vp, _vp, _vp, _vp, _vp]),
    "fpp_predict_mapped": (_c_int, [_vp, _vp, _c_int, _vp, _vp, _vp, _vp, _c_int, _vp]),
    "fpp_model_center_on": (_c_int, [_vp, _vp, _vp]),
    "fpp_update_matrices_QR": (_c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _dbl, _vp, _vp,
                                        _vp, _vp]),
    "fpp_pair_compute": (_c_int, [_vp, _i32, _i32, _vp, _vp, _i32, _vp, _vp, _vp,
                                  _c_int, _vp, _vp, _vp, _vp, _vp]),
    "fpp_model_set_L_inv": (_c_int, [_vp, _i32, _vp]),
    "fpp_likelihood_gradient_stable": (_c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp,
                                                _vp, _vp, _vp, _i32, _vp, _vp, _vp]),
    "fpp_model_set_max_memory": (_c_int, [_vp, _dbl]),
    "fpp_model_kuf_tiles": (_c_int, [_vp, _P(_i32), _P(_i32), _P(ctypes.c_float), _P(_i64)]),
    "fpp_model_pair_batches": (_c_int, [_vp, _P(_i32)]),
    "fpp_likelihood_gradient_stable_kernels": (_c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp,
                                                        _vp, _vp, _vp, _i32, _vp, _vp, _i32,
                                                        _vp, _vp, _vp]),
    "fpp_model_compute_varmap": (_c_int, [_vp, _vp, _vp]),
    "fpp_model_set_varmap": (_c_int, [_vp, _vp]),
    "fpp_std_atom_compute": (_c_int, [_vp, _i32, _i32, _vp, _vp, _i32, _vp, _vp, _vp,
                                      _i32, _vp, _vp]),
}

_lib = None


class FlareGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def lib():
    """Load the library once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FlareGpuError(FPP_ERR_UNSUPPORTED,
                            f"{LIB_PATH} is missing: run flare_pp_gb300.build.build()")
    l = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(l, name)
        fn.restype = res
        fn.argtypes = args
    _lib = l
    return l


def check(rc):
    if rc != FPP_OK:
        raise FlareGpuError(rc, lib().fpp_last_error().decode())
    return rc


def ptr(a):
    """Address of a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)
