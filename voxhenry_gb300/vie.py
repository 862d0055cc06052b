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

    def memory(self):
        """(bytes handed out, bytes cached) of the context's device block cache."""
        u, c = C.c_int64(), C.c_int64()
        _lib.check(self._lib.vh_ctx_memory(self.handle, C.byref(u), C.byref(c)), self.handle)
        return u.value, c.value

    def trim(self):
        """Frees the cached device blocks (after the context's queued work)."""
        _lib.check(self._lib.vh_ctx_trim(self.handle), self.handle)

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
        self._z0_real, self._z0_imag = z_real, (None if zi is None else z_imag)
        nc, nn, n = C.c_int64(), C.c_int64(), C.c_int64()
        _lib.check(lib.vh_geom_sizes(h, C.byref(nc), C.byref(nn), C.byref(n)), self.ctx.handle)
        self.n_curr, self.n_node, self.n = nc.value, nn.value, n.value

    @classmethod
    def generated(cls, L, M, N, dx, Ae, z_real, z_imag, idxS, want_fp32=False, ctx: Context | None = None):
        """Geometry whose circulant tensor fN_all2 is generated on the device.  Returns (geom, st2)."""
        g = cls.__new__(cls)
        g.ctx = ctx or default_context()
        lib = g.ctx._lib
        g.L, g.M, g.N, g.dx = int(L), int(M), int(N), float(dx)
        idx = np.ascontiguousarray(np.asarray(idxS, dtype=np.int64).ravel())
        A = sp.csc_matrix(Ae)
        A.sort_indices()
        jc = np.ascontiguousarray(A.indptr, dtype=np.int64)
        ir = np.ascontiguousarray(A.indices, dtype=np.int64)
        pr = np.ascontiguousarray(A.data, dtype=np.float64)
        zr = _fortran_flat(z_real, np.float64)
        zi = None if z_imag is None or np.size(z_imag) == 0 else _fortran_flat(z_imag, np.complex128)
        st2 = np.zeros(3, dtype=np.complex128)
        h = C.c_void_p()
        _lib.check(lib.vh_geom_create_generated(g.ctx.handle, g.L, g.M, g.N, g.dx, idx.size, _lib.i64ptr(idx),
                                                A.shape[0], _lib.i64ptr(jc), _lib.i64ptr(ir), _lib.dptr(pr),
                                                _lib.dptr(zr), _lib.cview(zi) if zi is not None else None,
                                                int(bool(want_fp32)), _lib.cview(st2), C.byref(h)), g.ctx.handle)
        g.handle = h
        g._z0_real, g._z0_imag = z_real, (None if zi is None else z_imag)
        nc, nn, n = C.c_int64(), C.c_int64(), C.c_int64()
        _lib.check(lib.vh_geom_sizes(h, C.byref(nc), C.byref(nn), C.byref(n)), g.ctx.handle)
        g.n_curr, g.n_node, g.n = nc.value, nn.value, n.value
        return g, st2

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

    def precon(self, st_sparse_precon, zslot=0, kind="schur_invert"):
        """lse_sparse_precon_prepare for this geometry (st already multiplied by j omega mu)."""
        return Precon(self, st_sparse_precon, zslot=zslot, kind=kind)

    def precons(self, st_list, zslots=None, kind="schur_invert"):
        """One preconditioner per frequency, factored together (vh_precon_create_batch)."""
        st = _lib.as_c128(np.asarray(st_list).reshape(-1, 3))
        F = st.shape[0]
        zs = np.zeros(F, dtype=np.int32) if zslots is None else np.ascontiguousarray(zslots, dtype=np.int32)
        hs = (C.c_void_p * F)()
        _lib.check(self.ctx._lib.vh_precon_create_batch(self.handle, PRECON_KIND[kind], F, _lib.cview(st),
                                                        zs.ctypes.data_as(C.POINTER(C.c_int)), hs), self.ctx.handle)
        return [Precon._from_handle(self, C.c_void_p(h), kind) for h in hs]

    def solve(self, b, pcs=None, scale=None, zslot=None, restart=50, tol=1e-8, maxit=10, flexible=False,
              prec="fp64", resvec_len=None, x0=None):
        """Batched pgmres / fpgmres from x0 (None: zero).  b, x0: (B, n).  Returns dict(x, flag, relres,
        iter, resvec)."""
        bb = _lib.as_c128(np.atleast_2d(b))
        B = bb.shape[0]
        if bb.shape[1] != self.n:
            raise ValueError(f"expected vectors of length {self.n}")
        if pcs is not None and not isinstance(pcs, (list, tuple)):
            pcs = [pcs] * B
        tolv = np.ascontiguousarray(np.broadcast_to(np.asarray(tol, dtype=np.float64), (B,)))
        s = None if scale is None else _lib.as_c128(np.broadcast_to(np.asarray(scale, dtype=np.complex128), (B,)))
        zs = None if zslot is None else np.ascontiguousarray(np.broadcast_to(zslot, (B,)), dtype=np.int32)
        rl = resvec_len or (restart * maxit + 1)
        x = _lib.host_empty(bb.shape, np.complex128)
        flag = np.zeros(B, dtype=np.int32)
        relres = np.zeros(B)
        it = np.zeros(2 * B, dtype=np.int32)
        resvec = np.zeros(B * rl)
        nres = np.zeros(B, dtype=np.int32)
        parr = None
        if pcs is not None:
            parr = (C.c_void_p * B)(*[p.handle for p in pcs])
        ip = C.POINTER(C.c_int)
        x0c = None
        if x0 is not None and np.count_nonzero(x0):
            x0c = _lib.as_c128(np.broadcast_to(np.asarray(x0, dtype=np.complex128), bb.shape))
        st = self.ctx._lib.vh_gmres_x0(self.handle, B, parr, _lib.cview(bb), _lib.cview(s) if s is not None else None,
                                       zs.ctypes.data_as(ip) if zs is not None else None, int(restart),
                                       _lib.dptr(tolv), int(maxit), int(bool(flexible)), _lib.PREC[prec],
                                       _lib.cview(x0c) if x0c is not None else None, _lib.cview(x),
                                       flag.ctypes.data_as(ip), _lib.dptr(relres), it.ctypes.data_as(ip),
                                       _lib.dptr(resvec), rl, nres.ctypes.data_as(ip))
        _lib.check(st, self.ctx.handle)
        rv = resvec.reshape(B, rl)
        return {"x": x, "flag": flag, "relres": relres, "iter": it.reshape(B, 2),
                "resvec": [rv[i, : min(rl, nres[i])].copy() for i in range(B)], "nres": nres}

    def close(self):
        if getattr(self, "handle", None):
            self.ctx._lib.vh_geom_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


PRECON_KIND = {"no_precond": 0, "schur_invert": 1, "schur_invert_df": 2, "schur_approx": 3, "schur_gmres": 4}


class Precon:
    """vh_precon: the state lse_sparse_precon_prepare leaves in MATLAB globals, on the device."""

    def __init__(self, geom: Geometry, st_sparse_precon, zslot=0, kind="schur_invert"):
        if kind not in PRECON_KIND:
            raise NotImplementedError(f"preconditioner '{kind}' is not available on the GPU path")
        self.geom = geom
        self.kind = kind
        st = _lib.as_c128(np.asarray(st_sparse_precon).ravel())
        if st.size != 3 and kind != "no_precond":
            raise ValueError("st_sparse_precon must hold 3 complex values")
        h = C.c_void_p()
        lib = geom.ctx._lib
        _lib.check(lib.vh_precon_create(geom.handle, PRECON_KIND[kind], _lib.cview(st) if st.size else None, zslot,
                                        C.byref(h)), geom.ctx.handle)
        self.handle = h

    @classmethod
    def _from_handle(cls, geom, handle, kind):
        p = cls.__new__(cls)
        p.geom, p.kind, p.handle = geom, kind, handle
        return p

    def stats(self):
        nnz, fl, nf, mf = C.c_int64(), C.c_double(), C.c_int(), C.c_int()
        _lib.check(self.geom.ctx._lib.vh_precon_stats(self.handle, C.byref(nnz), C.byref(fl), C.byref(nf), C.byref(mf)))
        return {"nnz_factor": nnz.value, "flops": fl.value, "fronts": nf.value, "max_front": mf.value}

    def set_prectol(self, prectol):
        """'schur_gmres': tolerance of the inner GMRES on S (lse_sparse_precon_multiply's prectol)."""
        _lib.check(self.geom.ctx._lib.vh_precon_set_prectol(self.handle, float(prectol)), self.geom.ctx.handle)
        return self

    def inner_iterations(self):
        """'schur_gmres': inner GMRES iterations summed over every apply so far."""
        t = C.c_int64()
        _lib.check(self.geom.ctx._lib.vh_precon_inner_iterations(self.handle, C.byref(t)), self.geom.ctx.handle)
        return t.value

    def apply(self, x):
        return apply_precons(self.geom, [self], x)

    __call__ = apply

    def close(self):
        if getattr(self, "handle", None):
            self.geom.ctx._lib.vh_precon_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def apply_precons(geom: Geometry, pcs, x):
    """Batched lse_sparse_precon_multiply: row b of x with pcs[b]."""
    x = np.asarray(x)
    single = x.ndim == 1
    xb = _lib.as_c128(x.reshape(1, -1) if single else x)
    B = xb.shape[0]
    if len(pcs) == 1 and B > 1:
        pcs = list(pcs) * B
    y = np.empty_like(xb)
    parr = (C.c_void_p * B)(*[p.handle for p in pcs])
    _lib.check(geom.ctx._lib.vh_precon_apply(geom.handle, B, parr, _lib.cview(xb), _lib.cview(y)), geom.ctx.handle)
    return y[0] if single else y


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


# ---------------------------------------------------------------------------------------------
# Preconditioner state of lse_sparse_precon_prepare / lse_sparse_precon_multiply.  The reference
# keeps it in MATLAB globals (lse_sparse_precon_prepare.m:2-3); here a module-level record holds
# the prepare arguments and the device factors built from them (one per geometry they are used on).
class _PreconState:
    def __init__(self, dx, z_real, z_imag, idxS, st, Ae, kind):
        self.dx, self.z_real, self.z_imag, self.idxS, self.st, self.Ae, self.kind = dx, z_real, z_imag, idxS, st, Ae, kind
        self.by_geom = {}
        self._own_geom = None

    def for_geometry(self, geom: Geometry) -> Precon:
        pc = self.by_geom.get(id(geom))
        if pc is None or pc.geom is not geom:
            slot = _z_slot_for(geom, self.z_real, self.z_imag)
            pc = Precon(geom, self.st, zslot=slot, kind=self.kind)
            self.by_geom[id(geom)] = pc
        return pc

    def own(self) -> Precon:
        if self._own_geom is None:
            L, M, N = np.shape(self.z_real)
            self._own_geom = _precon_only_geometry(self.Ae, self.z_real, self.z_imag, self.dx, self.idxS, (L, M, N))
        return self.for_geometry(self._own_geom)


_PRECON_STATE: _PreconState | None = None


def _z_slot_for(geom: Geometry, z_real, z_imag) -> int:
    """Slot of `geom` holding these z arrays (slot 0 is the creation z; others are added)."""
    slots = geom.__dict__.setdefault("_zslots", {0: (geom._z0_real, geom._z0_imag)})
    for s, (zr, zi) in slots.items():
        if zr is z_real and zi is z_imag:
            return s
    s = max(slots) + 1
    geom.set_z(s, z_real, z_imag)
    slots[s] = (z_real, z_imag)
    return s


def _precon_only_geometry(Ae, z_real, z_imag, dx, idxS, shape):
    g = Geometry.__new__(Geometry)
    g.ctx = default_context()
    lib = g.ctx._lib
    L, M, N = shape
    idx = np.ascontiguousarray(np.asarray(idxS, dtype=np.int64).ravel())
    A = sp.csc_matrix(Ae)
    A.sort_indices()
    jc = np.ascontiguousarray(A.indptr, dtype=np.int64)
    ir = np.ascontiguousarray(A.indices, dtype=np.int64)
    pr = np.ascontiguousarray(A.data, dtype=np.float64)
    zr = _fortran_flat(z_real, np.float64)
    zi = None if z_imag is None or np.size(z_imag) == 0 else _fortran_flat(z_imag, np.complex128)
    h = C.c_void_p()
    _lib.check(lib.vh_geom_create(g.ctx.handle, L, M, N, float(dx), None, idx.size, _lib.i64ptr(idx), A.shape[0],
                                  _lib.i64ptr(jc), _lib.i64ptr(ir), _lib.dptr(pr), _lib.dptr(zr),
                                  _lib.cview(zi) if zi is not None else None, 0, C.byref(h)), g.ctx.handle)
    g.handle = h
    g.L, g.M, g.N, g.dx = L, M, N, float(dx)
    g._z0_real, g._z0_imag = z_real, z_imag
    nc, nn, n = C.c_int64(), C.c_int64(), C.c_int64()
    _lib.check(lib.vh_geom_sizes(h, C.byref(nc), C.byref(nn), C.byref(n)), g.ctx.handle)
    g.n_curr, g.n_node, g.n = nc.value, nn.value, n.value
    return g


def lse_sparse_precon_prepare(dx, z_real, z_imag, idxS, st_sparse_precon, nodeid_4_grnd=None,
                              nodeid_4_injectcurr=None, Ae=None, kind="schur_invert"):
    """lse_sparse_precon_prepare.m:1 -- no outputs; the factor is kept as module state."""
    global _PRECON_STATE
    if kind not in PRECON_KIND:
        raise NotImplementedError(f"preconditioner '{kind}' is not available on the GPU path")
    _PRECON_STATE = _PreconState(float(dx), z_real, None if z_imag is None or np.size(z_imag) == 0 else z_imag,
                                 np.asarray(idxS).ravel(), np.asarray(st_sparse_precon).ravel(), Ae, kind)


def lse_sparse_precon_multiply(JOut_full_in, Ae=None, nodeid_4_grnd=None, nodeid_4_injectcurr=None, prectol=None):
    """lse_sparse_precon_multiply.m:1 -- applies the prepared preconditioner ('schur_gmres' uses
    prectol, the inner tolerance; None keeps the handle's, 0.1 by default)."""
    if _PRECON_STATE is None:
        raise RuntimeError("lse_sparse_precon_prepare has not been called")
    pc = _PRECON_STATE.own()
    if prectol is not None and pc.kind == "schur_gmres":
        pc.set_prectol(prectol)
    return pc.apply(np.asarray(JOut_full_in).ravel())


class MatvecHandle:
    """@(J) lse_matvect_mult(J, fN_all, Ae, z_real, z_imag, dx, idxS5, ...) bound to the device."""

    def __init__(self, fN_all, Ae, z_real, z_imag, dx, idx, prec="fp64"):
        self.geom = _cached_geometry(fN_all, Ae, z_real, z_imag, dx, idx, prec)
        self.geom.__dict__.setdefault("_z0_real", z_real)
        self.geom.__dict__.setdefault("_z0_imag", None if z_imag is None or np.size(z_imag) == 0 else z_imag)
        self.prec = prec

    def __call__(self, J):
        return self.geom.matvec(np.asarray(J).ravel(), prec=self.prec)


def matvec_handle(fN_all, Ae, z_real, z_imag, dx, idx, nodeid_4_grnd=None, nodeid_4_injectcurr=None, prec="fp64"):
    return MatvecHandle(fN_all, Ae, z_real, z_imag, dx, idx, prec)


class PreconHandle:
    """@(x) lse_sparse_precon_multiply(x, ...) bound to the current prepared state."""

    def __init__(self):
        if _PRECON_STATE is None:
            raise RuntimeError("lse_sparse_precon_prepare has not been called")
        self.state = _PRECON_STATE

    def __call__(self, x):
        return self.state.own().apply(np.asarray(x).ravel())


def precon_handle():
    return PreconHandle()


def _resolve_precon(op, geom):
    if op is None:
        return None
    if isinstance(op, PreconHandle):
        return op.state.for_geometry(geom)
    if op is lse_sparse_precon_multiply:
        if _PRECON_STATE is None:
            raise RuntimeError("lse_sparse_precon_prepare has not been called")
        return _PRECON_STATE.for_geometry(geom)
    if isinstance(op, Precon):
        if op.geom is not geom:
            raise ValueError("the preconditioner belongs to another geometry")
        return op
    raise TypeError("the GPU pgmres takes the preconditioner as precon_handle() / lse_sparse_precon_multiply")


def _krylov(A, b, restart, tol, maxit, P, flexible, x0, prec):
    if not isinstance(A, MatvecHandle):
        # iterchk.m:16-43 also takes a matrix A (and matrix preconditioners, applied as L1 \ x): the
        # GPU solver is built for the VIE operator of lse_matvect_mult and its Schur preconditioner only
        raise TypeError("the GPU pgmres takes the operator as matvec_handle(...) (lse_matvect_mult's arguments); "
                        "matrix operators (iterchk.m:16-43) are not supported")
    g = A.geom
    pc = _resolve_precon(P, g)
    b = np.asarray(b).ravel()
    x0v = None if x0 is None else np.asarray(x0, dtype=np.complex128).ravel()
    if x0v is not None and x0v.size != b.size:
        raise ValueError("x0 must have the length of b")
    out = g.solve(b[None, :], pcs=None if pc is None else [pc], restart=restart, tol=tol, maxit=maxit,
                  flexible=flexible, prec=prec if prec else A.prec, x0=None if x0v is None else x0v[None, :])
    it = out["iter"][0]
    return out["x"][0], int(out["flag"][0]), float(out["relres"][0]), (int(it[0]), int(it[1])), out["resvec"][0]


def pgmres(A, b, restart=50, tol=1e-3, maxit=10, L1=None, L2=None, R1=None, R2=None, x0=None, prec=None):
    """[x, flag, relres, iter, resvec] = pgmres(A, b, restart, tol, maxit, L1, L2, R1, R2, x0)  (pgmres.m:70).

    A: matvec_handle(...).  One preconditioner, precon_handle() or lse_sparse_precon_multiply: on the left
    as L1 (the executer's form, VoxHenry_executer.m:294-295), or on the right as R1 (right-preconditioned
    GMRES: the flexible solver with a fixed preconditioner, whose iterates are the same).  x0: initial
    guess (None or zeros: x0 = 0).  A second preconditioner (L1 with L2, R1 or R2) is not supported:
    the executer never passes one."""
    given = [k for k, v in (("L1", L1), ("L2", L2), ("R1", R1), ("R2", R2)) if v is not None]
    if len(given) > 1 or given in (["L2"], ["R2"]):
        raise NotImplementedError(f"one preconditioner, L1 or R1, is supported (got {', '.join(given)})")
    if given == ["R1"]:
        return _krylov(A, b, restart, tol, maxit, R1, True, x0, prec)
    return _krylov(A, b, restart, tol, maxit, L1, False, x0, prec)


def fpgmres(A, b, restart=50, tol=1e-3, maxit=10, R1=None, R2=None, x0=None):
    """[x, flag, relres, iter, resvec] = fpgmres(A, b, restart, tol, maxit, R1, R2, x0)  (fpgmres.m:58)."""
    if R2 is not None:
        raise NotImplementedError("one right preconditioner (R1) is supported")
    return _krylov(A, b, restart, tol, maxit, R1, True, x0, "fp64")
