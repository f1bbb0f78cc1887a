"""ctypes binding of libtennet_cuda.so (the C ABI declared in include/tennet.h).

The library is the only compute path: if it is missing, loading fails with an error that
says how to build it.  There is no host fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libtennet_cuda.so")

TN_OK = 0
TN_E_INVALID = -1
TN_E_CUDA = -2
TN_E_NOMEM = -3
TN_E_NOTCONV = -4
TN_E_NOGPU = -5
TN_E_TIMEOUT = -6
TN_PREC_FP64 = 0
TN_PREC_SPLIT = 1
TN_ORTHO_LEFT = 0
TN_ORTHO_RIGHT = 1

i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)
vp = C.c_void_p


class UpdateParams(C.Structure):
    _fields_ = [
        ("maxdim", C.c_int32),
        ("mindim", C.c_int32),
        ("cutoff", C.c_double),
        ("normalize", C.c_int32),
        ("krylovdim", C.c_int32),
        ("maxiter", C.c_int32),
        ("tol", C.c_double),
        ("eager", C.c_int32),
        ("check_convergence", C.c_int32),
        ("noise", C.c_double),
    ]


class UpdateResult(C.Structure):
    _fields_ = [
        ("energy", C.c_double),
        ("truncerr", C.c_double),
        ("newdim", C.c_int32),
        ("matvecs", C.c_int32),
        ("converged", C.c_int32),
        ("neigs", C.c_int32),
    ]


class SweepResult(C.Structure):
    _fields_ = [
        ("energy", C.c_double),
        ("maxtruncerr", C.c_double),
        ("maxlinkdim", C.c_int32),
        ("matvecs", C.c_int32),
        ("heff_flops", C.c_double),
        ("heff_ms", C.c_double),
        ("env_ms", C.c_double),
        ("svd_ms", C.c_double),
        ("lanczos_ms", C.c_double),
        ("sweep_ms", C.c_double),
        ("gemm_ms", C.c_double),
        ("gemm_flops", C.c_double),
        ("pack_ms", C.c_double),
        ("gemm_launches", C.c_int64),
        ("kernel_launches", C.c_int64),
        ("qr_panel_ms", C.c_double),
        ("qr_gemm_ms", C.c_double),
        ("krylov_bytes", C.c_double),
        ("svd_gemm_flops", C.c_double),
        ("svd_jacobi_flops", C.c_double),
        ("svd_sweeps32", C.c_int32),
        ("svd_sweeps_df", C.c_int32),
        ("svd_small_flops", C.c_double),
    ]


# name -> (restype, argtypes)
PROTOS = {
    "tn_ctx_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
    "tn_ctx_destroy": (C.c_int, [vp]),
    "tn_ctx_set_precision": (C.c_int, [vp, C.c_int, C.c_int]),
    "tn_ctx_set_svd_split": (C.c_int, [vp, C.c_int]),
    "tn_ctx_svd_schedule": (C.c_int, [vp, C.POINTER(C.c_int32), C.POINTER(C.c_float), C.c_int,
                                      C.POINTER(C.c_int)]),
    "tn_ctx_inject_wait_timeout": (C.c_int, [vp, C.c_int]),
    "tn_last_error": (C.c_char_p, []),
    "tn_version": (C.c_char_p, []),
    "tn_kernel_launches": (C.c_int64, []),
    "tn_mpo_create": (C.c_int, [vp, C.c_int, C.c_int, i32p, i32p, i32p, f64p, C.POINTER(vp)]),
    "tn_mpo_destroy": (C.c_int, [vp]),
    "tn_mps_create": (C.c_int, [vp, C.c_int, C.c_int, i32p, i32p, i32p, i32p, f64p, C.c_int,
                                C.POINTER(vp)]),
    "tn_mps_create_complex": (C.c_int, [vp, C.c_int, C.c_int, i32p, i32p, i32p, i32p, f64p,
                                        C.c_int, C.POINTER(vp)]),
    "tn_mps_create_blocks": (C.c_int, [vp, C.c_int, C.c_int, i32p, i32p, i32p, i32p, f64p,
                                       C.POINTER(C.c_int64), C.c_int, C.POINTER(vp)]),
    "tn_mps_site_blocks": (C.c_int, [vp, C.c_int, f64p, C.c_int64, C.POINTER(C.c_int64)]),
    "tn_mps_destroy": (C.c_int, [vp]),
    "tn_mps_link": (C.c_int, [vp, C.c_int, i32p, i32p, i32p, C.c_int]),
    "tn_mps_site": (C.c_int, [vp, C.c_int, f64p, C.c_int64]),
    "tn_mps_center": (C.c_int, [vp]),
    "tn_mps_make_complex": (C.c_int, [vp]),
    "tn_mps_is_complex": (C.c_int, [vp]),
    "tn_mps_site_complex": (C.c_int, [vp, C.c_int, f64p, C.c_int64]),
    "tn_mps_overlap_complex": (C.c_int, [vp, vp, f64p]),
    "tn_mps_expect_local": (C.c_int, [vp, f64p, f64p]),
    "tn_mps_overlap": (C.c_int, [vp, vp, f64p]),
    "tn_env_create": (C.c_int, [vp, vp, C.POINTER(vp)]),
    "tn_env_set_projectors": (C.c_int, [vp, C.POINTER(vp), C.c_int, C.c_double]),
    "tn_env_destroy": (C.c_int, [vp]),
    "tn_env_getpsi": (C.c_int, [vp, C.POINTER(vp)]),
    "tn_env_position": (C.c_int, [vp, C.c_int, C.c_int]),
    "tn_env_product": (C.c_int, [vp, f64p, f64p, C.c_int64]),
    "tn_env_product_complex": (C.c_int, [vp, f64p, f64p, C.c_int64]),
    "tn_env_make_complex": (C.c_int, [vp]),
    "tn_env_environment": (C.c_int, [vp, C.c_int, C.c_int, f64p, C.c_int64, i32p]),
    "tn_env_product_flops": (C.c_int, [vp, f64p]),
    "tn_env_update_position": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(UpdateParams),
                                         C.POINTER(UpdateResult), f64p, C.c_int]),
    "tn_env_fullsweep": (C.c_int, [vp, C.POINTER(UpdateParams), C.POINTER(SweepResult), f64p,
                                   C.c_int, i32p]),
    "tn_env_update_position_nsite": (C.c_int, [vp, C.c_int, C.c_int, C.c_int,
                                               C.POINTER(UpdateParams), C.POINTER(UpdateResult),
                                               f64p, C.c_int]),
    "tn_env_fullsweep_nsite": (C.c_int, [vp, C.c_int, C.POINTER(UpdateParams),
                                         C.POINTER(SweepResult), f64p, C.c_int, i32p]),
    "tn_env_tdvpsweep": (C.c_int, [vp, C.c_double, C.POINTER(UpdateParams), C.POINTER(SweepResult),
                                   f64p, C.c_int, i32p]),
    "tn_env_tdvpsweep_complex": (C.c_int, [vp, C.c_double, C.c_double, C.POINTER(UpdateParams),
                                           C.POINTER(SweepResult), f64p, C.c_int, i32p]),
    "tn_env_tdvpsweep_nsite": (C.c_int, [vp, C.c_int, C.c_double, C.c_double,
                                         C.POINTER(UpdateParams), C.POINTER(SweepResult), f64p,
                                         C.c_int, i32p]),
    "tn_env_fullsweep_dynamic": (C.c_int, [vp, C.c_double, f64p, i32p, C.POINTER(UpdateParams),
                                           C.POINTER(SweepResult), f64p, C.c_int, i32p]),
    "tn_env_tdvpsweep_dynamic": (C.c_int, [vp, C.c_double, C.c_double, C.c_double, f64p, i32p,
                                           C.POINTER(UpdateParams), C.POINTER(SweepResult), f64p,
                                           C.c_int, i32p]),
    "tn_env_bond_spectra": (C.c_int, [vp, f64p, C.c_int64, i32p, C.c_int]),
    "tn_env_update_mpo": (C.c_int, [vp, vp, C.c_int]),
    "tn_svd_truncate": (C.c_int, [vp, C.c_int, i32p, i32p, f64p, C.c_int32, C.c_int32,
                                  C.c_double, i32p, f64p, f64p]),
    "tn_block_svals_noalloc": (C.c_int, [C.c_int, vp, C.c_int, i32p, i32p, vp, vp]),
    "tn_ttn_create": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, i32p, i32p, i32p, f64p,
                                C.c_int, C.POINTER(vp)]),
    "tn_ttn_destroy": (C.c_int, [vp]),
    "tn_ttn_center": (C.c_int, [vp]),
    "tn_ttn_node_dims": (C.c_int, [vp, C.c_int, i32p, i32p]),
    "tn_ttn_node": (C.c_int, [vp, C.c_int, f64p, C.c_int64]),
    "tn_ttn_maxlinkdim": (C.c_int, [vp]),
    "tn_ttn_isometrize": (C.c_int, [vp, C.c_int, C.c_int]),
    "tn_ttn_model_create": (C.c_int, [C.c_int, C.c_int, C.c_int, i32p, i32p, f64p, f64p,
                                      C.POINTER(vp)]),
    "tn_ttn_model_destroy": (C.c_int, [vp]),
    "tn_ttn_envs_create": (C.c_int, [C.c_int, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "tn_ttn_env_destroy": (C.c_int, [vp]),
    "tn_ttn_env_getpsi": (C.c_int, [vp, C.POINTER(vp)]),
    "tn_ttn_env_center": (C.c_int, [vp]),
    "tn_ttn_env_position": (C.c_int, [vp, C.c_int]),
    "tn_ttn_env_product": (C.c_int, [vp, f64p, f64p, C.c_int64]),
    "tn_ttn_env_product_flops": (C.c_int, [vp, f64p]),
    "tn_ttn_env_set_projectors": (C.c_int, [vp, C.POINTER(vp), C.c_int, C.c_double]),
    "tn_ttn_env_update_position": (C.c_int, [vp, C.c_int, C.POINTER(UpdateParams),
                                             C.POINTER(UpdateResult)]),
    "tn_ttn_envs_fullsweep": (C.c_int, [C.c_int, C.POINTER(vp), C.c_int, i32p,
                                        C.POINTER(UpdateParams), C.POINTER(SweepResult)]),
    "tn_ttn_envs_fullsweep_expand": (C.c_int, [C.c_int, C.POINTER(vp), C.c_int, i32p, C.c_int,
                                               C.POINTER(UpdateParams), C.c_int, C.c_int,
                                               C.c_int, C.c_uint64, C.POINTER(SweepResult)]),
}

_lib = None


class TenNetError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def load(path: str | None = None):
    """Load libtennet_cuda.so and bind every exported symbol of tennet.h."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    for name, (res, args) in PROTOS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(code):
    if code != TN_OK:
        msg = load().tn_last_error().decode(errors="replace")
        if code == TN_E_NOTCONV:
            raise TenNetError(code, msg)
        raise TenNetError(code, msg)
    return code


def as_i32(a):
    import numpy as np
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(i32p)


def as_f64(a):
    import numpy as np
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(f64p)
