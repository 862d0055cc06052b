"""ctypes binding of libvhgpu.so (declarations mirror include/voxhenry_gpu.h).

The library is required: there is no CPU fallback.  Loading fails loudly when
libvhgpu.so is missing (build it with ``voxhenry_gb300._build.build()``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libvhgpu.so")

VH_OK = 0
VH_ERR_OOM = 2
STATUS = {0: "VH_OK", 1: "VH_ERR_BAD_ARG", 2: "VH_ERR_OOM", 3: "VH_ERR_UNSUPPORTED", 4: "VH_ERR_TIMEOUT",
          5: "VH_ERR_NOT_CONVERGED", 6: "VH_ERR_CUDA", 7: "VH_ERR_NO_DEVICE"}
PREC = {"fp64": 0, "fp32": 1, "df": 2}

_p = C.c_void_p
_i64p = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

# name -> (restype, argtypes)
SIGNATURES = {
    "vh_version": (C.c_int, []),
    "vh_status_string": (C.c_char_p, [C.c_int]),
    "vh_ctx_create": (C.c_int, [C.c_int, C.POINTER(_p)]),
    "vh_ctx_destroy": (None, [_p]),
    "vh_last_error": (C.c_char_p, [_p]),
    "vh_ctx_synchronize": (C.c_int, [_p]),
    "vh_ctx_memory": (C.c_int, [_p, _i64p, _i64p]),
    "vh_ctx_trim": (C.c_int, [_p]),
    "vh_geom_create": (C.c_int, [_p, C.c_int, C.c_int, C.c_int, C.c_double, _dp, C.c_int64, _i64p, C.c_int64,
                                 _i64p, _i64p, _dp, _dp, _dp, C.c_int, C.POINTER(_p)]),
    "vh_geom_destroy": (None, [_p]),
    "vh_geom_sizes": (C.c_int, [_p, _i64p, _i64p, _i64p]),
    "vh_geom_set_z": (C.c_int, [_p, C.c_int, _dp, _dp]),
    "vh_matvec": (C.c_int, [_p, C.c_int, _dp, _dp, _dp, _ip, C.c_int]),
    "vh_matvec_device": (C.c_int, [_p, C.c_int, _p, _p, _p, _ip, C.c_int]),
    "vh_matvec_device_noalloc": (C.c_int, [_p, C.c_int, _p, _p, _p, _ip, C.c_int]),
    "vh_conv_tune": (C.c_int, [_p, C.c_int, C.c_int, _ip, _ip, _ip, _ip, _dp]),
    "vh_conv_set_tuning": (C.c_int, [_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "vh_currents_on_grid": (C.c_int, [_p, C.c_int, C.c_int, C.c_int, C.c_int64, _i64p, C.c_int, _dp, C.c_int64, _dp]),
    "vh_sparse_matvec": (C.c_int, [_p, C.c_int64, C.c_int64, _i64p, _i64p, _dp, C.c_int, _dp, C.c_int64, _dp, C.c_int64]),
    "vh_precon_create": (C.c_int, [_p, C.c_int, _dp, C.c_int, C.POINTER(_p)]),
    "vh_precon_destroy": (None, [_p]),
    "vh_precon_create_batch": (C.c_int, [_p, C.c_int, C.c_int, _dp, _ip, C.POINTER(_p)]),
    "vh_precon_stats": (C.c_int, [_p, _i64p, _dp, _ip, _ip]),
    "vh_precon_set_prectol": (C.c_int, [_p, C.c_double]),
    "vh_precon_inner_iterations": (C.c_int, [_p, _i64p]),
    "vh_schur_analyze": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int64, _i64p, C.c_int64, _i64p, _i64p, _dp,
                                   _i64p, _dp, _ip, _ip, _i64p]),
    "vh_precon_apply": (C.c_int, [_p, C.c_int, C.POINTER(_p), _dp, _dp]),
    "vh_precon_apply_device": (C.c_int, [_p, C.c_int, C.POINTER(_p), _p, _p]),
    "vh_geom_create_generated": (C.c_int, [_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int64, _i64p, C.c_int64,
                                           _i64p, _i64p, _dp, _dp, _dp, C.c_int, _dp, C.POINTER(_p)]),
    "vh_panel_ids": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int64, _i64p, _i64p, _i64p]),
    "vh_incidence": (C.c_int, [C.c_int64, _i64p, _i64p, _i64p, _dp]),
    "vh_setup_device": (C.c_int, [_p, C.c_int, C.c_int, C.c_int, C.c_int64, _i64p, _i64p, _i64p, _i64p, _i64p,
                                  _dp]),
    "vh_circulant_tensor": (C.c_int, [_p, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp]),
    "vh_gmres_device": (C.c_int, [_p, C.c_int, C.POINTER(_p), _p, _dp, _ip, C.c_int, _dp, C.c_int, C.c_int, C.c_int,
                                  _p, _ip, _dp, _ip, _dp, C.c_int, _ip]),
    "vh_ctx_stream": (C.c_void_p, [_p]),
    "vh_ctx_profile": (C.c_int, [_p, C.c_int]),
    "vh_ctx_profile_read": (C.c_int, [_p, _dp, _i64p, _i64p, C.c_int]),
    "vh_launch_count": (C.c_int64, []),
    "vh_gmres": (C.c_int, [_p, C.c_int, C.POINTER(_p), _dp, _dp, _ip, C.c_int, _dp, C.c_int, C.c_int, C.c_int, _dp,
                           _ip, _dp, _ip, _dp, C.c_int, _ip]),
    "vh_gmres_x0": (C.c_int, [_p, C.c_int, C.POINTER(_p), _dp, _dp, _ip, C.c_int, _dp, C.c_int, C.c_int, C.c_int, _dp,
                              _dp, _ip, _dp, _ip, _dp, C.c_int, _ip]),
    "vh_gmres_device_x0": (C.c_int, [_p, C.c_int, C.POINTER(_p), _p, _dp, _ip, C.c_int, _dp, C.c_int, C.c_int, C.c_int,
                                     _p, _p, _ip, _dp, _ip, _dp, C.c_int, _ip]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libvhgpu.so and declare every exported entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with voxhenry_gb300._build.build() (requires nvcc)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class VHError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def check(status: int, ctx=None):
    if status != VH_OK:
        lib = load()
        msg = lib.vh_last_error(ctx).decode() if ctx else lib.vh_status_string(status).decode()
        raise VHError(status, msg)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp) if a is not None else None


def i64ptr(a: np.ndarray):
    return a.ctypes.data_as(_i64p) if a is not None else None


def as_c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def host_empty(shape, dtype=np.complex128) -> np.ndarray:
    """An uninitialised host array in page-locked memory when a GPU is present, so that the
    library's host<->device copies of it run as direct DMA; a plain array otherwise.  The memory
    comes from torch's caching host allocator (the array keeps its tensor alive)."""
    try:
        import torch

        if torch.cuda.is_available():
            nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
            t = torch.empty(max(nbytes, 1), dtype=torch.uint8, pin_memory=True)
            return t.numpy()[:nbytes].view(dtype).reshape(shape)
    except ImportError:
        pass
    return np.empty(shape, dtype=dtype)


def as_f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def cview(a: np.ndarray):
    """complex128 array -> pointer to interleaved doubles."""
    return a.ctypes.data_as(_dp)
