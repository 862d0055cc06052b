"""Autotuning of the FFT convolution's launch choices, with a cache on disk.

The FFT convolution of lse_matvect_mult.m:57-93 has launch choices whose best setting depends on the
grid, the voxel box, the precision and the batch width: the y-pass (the register pass for padded y
lengths 256, 512, 1024 over 128- or 64-byte rows, or the shared-memory Stockham pass), the z-pass (two
lanes per column, one thread per column for padded z lengths up to 32, or the direct Toeplitz
convolution for voxel boxes up to 16 rows), the x passes (complex64: one warp per line for padded x
lengths 256, 512, 1024) and how many right-hand sides share one launch sequence.  vh_conv_tune times the candidates on the geometry itself with CUDA events; the
choice is cached in a JSON file keyed by the GPU, the library build (the digest of the sources its
kernels were compiled from: a rebuilt library times its choices again), the grid, the voxel box, the
precision and the batch width, so later runs (and other geometries of the same shape) apply it
without timing.

Cache file: $VOXHENRY_TUNE_CACHE, else ~/.cache/voxhenry_gb300/conv_tuning.json.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import threading

from . import _build, _lib

PREC = _lib.PREC
_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("VOXHENRY_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "voxhenry_gb300",
                                                                   "conv_tuning.json")


def device_name() -> str:
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except ImportError:
        pass
    return "unknown"


def tuning_key(grid, box, prec: str, B: int, device: str | None = None, lib: str | None = None) -> str:
    """grid: (L, M, N); box: (ny, nz) voxel box of the FFT passes; B: right-hand sides per call
    (rounded up to a power of two: nearby batch widths share a choice); lib: the library build
    (default: the one in the package)."""
    b = 1
    while b < B:
        b *= 2
    return (f"{device or device_name()}|lib={lib or _build.build_id()}|grid={grid[0]}x{grid[1]}x{grid[2]}"
            f"|box={box[0]}x{box[1]}|{prec}|B<={b}")


def load_cache(path: str | None = None) -> dict:
    p = path or cache_path()
    try:
        with open(p) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def store(key: str, choice: dict, path: str | None = None) -> None:
    p = path or cache_path()
    with _lock:
        d = load_cache(p)
        d[key] = choice
        os.makedirs(os.path.dirname(p) or ".", exist_ok=True)
        tmp = p + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)


def box_of(prob) -> tuple:
    """(ny, nz): the y and z extent of the voxels, the rows the FFT passes visit."""
    import numpy as np

    idx = np.asarray(prob.idxS).ravel() - 1
    j = (idx // prob.L) % prob.M
    k = idx // (prob.L * prob.M)
    return int(j.max() - j.min() + 1), int(k.max() - k.min() + 1)


def tune(geom, prec: str, B: int, grid, box, path: str | None = None, retune: bool = False, timer=None) -> dict:
    """Applies the cached choice for this (grid, box, prec, B) to `geom`, or times the candidates
    (vh_conv_tune, or `timer(geom, prec, B)` in tests) and caches the winner.  Returns the choice
    {"y_variant", "z_variant", "max_rhs", "x_variant", "ms_per_rhs", "cached"}."""
    key = tuning_key(grid, box, prec, B)
    if not retune:
        hit = load_cache(path).get(key)
        if hit is not None:
            _set(geom, prec, hit["y_variant"], hit.get("z_variant", 0), hit["max_rhs"], hit.get("x_variant", 0))
            return dict(hit, cached=True)
    if timer is not None:
        choice = timer(geom, prec, B)
    else:
        yv, zv, mr, xv, ms = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_double()
        _lib.check(geom.ctx._lib.vh_conv_tune(geom.handle, PREC[prec], int(B), C.byref(yv), C.byref(zv), C.byref(mr),
                                              C.byref(xv), C.byref(ms)), geom.ctx.handle)
        choice = {"y_variant": yv.value, "z_variant": zv.value, "max_rhs": mr.value, "x_variant": xv.value,
                  "ms_per_rhs": ms.value}
    store(key, choice, path)
    return dict(choice, cached=False)


def _set(geom, prec, y_variant, z_variant, max_rhs, x_variant=0):
    if hasattr(geom, "ctx"):
        _lib.check(geom.ctx._lib.vh_conv_set_tuning(geom.handle, PREC[prec], int(y_variant), int(z_variant),
                                                    int(max_rhs), int(x_variant)), geom.ctx.handle)
    else:   # a stand-in geometry (tests)
        geom.tuning = (prec, y_variant, z_variant, max_rhs, x_variant)
