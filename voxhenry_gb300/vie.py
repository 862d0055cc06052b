"""Host-side mirror of the reference's solve-path calls, backed by libvhgpu.so.

    lse_matvect_mult(JIn0, fN_all, Ae, z_real, z_imag, dx, idx, nodeid_4_grnd, nodeid_4_injectcurr)
        src_lse_formation/lse_matvect_mult.m:1 -- same arguments, same result.

Arrays follow the reference's MATLAB conventions: 3-D/4-D arrays are
column-major (x fastest), ``idx`` (idxS5) holds 1-based linear indices, Ae is a
SciPy sparse matrix with the port rows already removed.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import _lib


class Context:
    """One CUDA device and stream (vh_ctx)."""

    def __init__(self, device: int = 0):
        self._lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self._lib.vh_ctx_create(device, C.byref(h)))
        self.handle = h

    def synchronize(self):
        _lib.check(self._lib.vh_ctx_synchronize(self.handle), self.handle)

    def close(self):
        if self.handle:
            self._lib.vh_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _fortran_flat(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype).ravel(order="F"))


class Geometry:
    """Device-resident fixed arguments of lse_matvect_mult (vh_geom)."""

    def __init__(self, fN_all, Ae, z_real, z_imag, dx, idxS, want_fp32=False, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        lib = self.ctx._lib
        fN_all = np.asarray(fN_all)
        X, Y, Z, K = fN_all.shape
        if K != 7 or X % 2 or Y % 2 or Z % 2:
            raise ValueError("fN_all must have shape (2L, 2M, 2N, 7)")
        L, M, N = X // 2, Y // 2, Z // 2
        self.L, self.M, self.N = L, M, N
        self.dx = float(dx)
        fn = _fortran_flat(fN_all, np.complex128)
        idxS = np.ascontiguousarray(np.asarray(idxS, dtype=np.int64).ravel())
        A = sp.csc_matrix(Ae)
        A.sort_indices()
        jc = np.ascontiguousarray(A.indptr, dtype=np.int64)
        ir = np.ascontiguousarray(A.indices, dtype=np.int64)
        pr = np.ascontiguousarray(A.data, dtype=np.float64)
        if A.shape[1] != 5 * idxS.size:
            raise ValueError("Ae must have 5*nv columns")
        zr = _fortran_flat(z_real, np.float64)
        zi = None if z_imag is None or np.size(z_imag) == 0 else _fortran_flat(z_imag, np.complex128)
        h = C.c_void_p()
        st = lib.vh_geom_create(self.ctx.handle, L, M, N, self.dx, _lib.cview(fn), idxS.size, _lib.i64ptr(idxS),
                                A.shape[0], _lib.i64ptr(jc), _lib.i64ptr(ir), _lib.dptr(pr), _lib.dptr(zr),
                                _lib.cview(zi) if zi is not None else None, int(bool(want_fp32)), C.byref(h))
        _lib.check(st, self.ctx.handle)
        self.handle = h
        nc, nn, n = C.c_int64(), C.c_int64(), C.c_int64()
        _lib.check(lib.vh_geom_sizes(h, C.byref(nc), C.byref(nn), C.byref(n)), self.ctx.handle)
        self.n_curr, self.n_node, self.n = nc.value, nn.value, n.value

    def set_z(self, slot, z_real, z_imag=None):
        zr = _fortran_flat(z_real, np.float64)
        zi = None if z_imag is None else _fortran_flat(z_imag, np.complex128)
        _lib.check(self.ctx._lib.vh_geom_set_z(self.handle, slot, _lib.dptr(zr), _lib.cview(zi) if zi is not None else None),
                   self.ctx.handle)

    def matvec(self, x, scale=None, zslot=None, prec="fp64"):
        """y = A x for one (n,) or a batch (B, n) of right-hand sides."""
        x = np.asarray(x)
        single = x.ndim == 1
        xb = _lib.as_c128(x.reshape(1, -1) if single else x)
        if xb.shape[1] != self.n:
            raise ValueError(f"expected vectors of length {self.n}")
        B = xb.shape[0]
        y = np.empty_like(xb)
        s = None if scale is None else _lib.as_c128(np.broadcast_to(np.asarray(scale, dtype=np.complex128), (B,)))
        zs = None if zslot is None else np.ascontiguousarray(np.broadcast_to(zslot, (B,)), dtype=np.int32)
        st = self.ctx._lib.vh_matvec(self.handle, B, _lib.cview(xb), _lib.cview(y),
                                     _lib.cview(s) if s is not None else None,
                                     zs.ctypes.data_as(C.POINTER(C.c_int)) if zs is not None else None,
                                     _lib.PREC[prec])
        _lib.check(st, self.ctx.handle)
        return y[0] if single else y

    def close(self):
        if getattr(self, "handle", None):
            self.ctx._lib.vh_geom_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# Geometry cache of the drop-in call: MATLAB keeps fN_all / Ae / z stable across the
# anonymous-function calls of one frequency (VoxHenry_executer.m:287-290); so do callers here.
_geom_cache: dict = {}


def _cached_geometry(fN_all, Ae, z_real, z_imag, dx, idx, prec):
    key = (id(fN_all), id(Ae), id(z_real), id(z_imag), float(dx), id(idx))
    ent = _geom_cache.get(key)
    if ent is None or ent[1] is not fN_all or (prec == "fp32" and not ent[2]):
        nv = np.asarray(idx).size // 5
        g = Geometry(fN_all, Ae, z_real, z_imag, dx, np.asarray(idx).ravel()[:nv], want_fp32=(prec == "fp32"))
        if len(_geom_cache) > 8:
            _geom_cache.clear()
        ent = (g, fN_all, prec == "fp32", Ae, z_real, z_imag, idx)
        _geom_cache[key] = ent
    return ent[0]


def lse_matvect_mult(JIn0, fN_all, Ae, z_real, z_imag, dx, idx, nodeid_4_grnd=None, nodeid_4_injectcurr=None,
                     prec="fp64"):
    """JOut_full = lse_matvect_mult(JIn0, fN_all, Ae, z_real, z_imag, dx, idx, nodeid_4_grnd, nodeid_4_injectcurr).

    lse_matvect_mult.m:1-140.  ``nodeid_4_grnd``/``nodeid_4_injectcurr`` only matter for the
    'schur_invert_original' layout, which keeps zeroed port rows; the GPU path takes Ae with the
    port rows removed (the executer's default), so they are accepted and ignored.
    """
    g = _cached_geometry(fN_all, Ae, z_real, z_imag, dx, idx, prec)
    return g.matvec(np.asarray(JIn0).ravel(), prec=prec)
