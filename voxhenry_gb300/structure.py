"""Problem setup of VoxHenry_executer.m:69-200 on the product side.

Panel numbering and the incidence matrix come from the native builders (vh_panel_ids,
vh_incidence); the circulant tensor is generated on the device (vh_geom_create_generated /
vh_circulant_tensor).  Port handling follows lse_assign_exc_grnd_nodes.m:1-94 and
VoxHenry_executer.m:159-193 (RHS = -sum of the injection rows of Ae, then the port rows are
removed from Ae and from the RHS).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import _lib
from .executer import Problem


def nonempty_voxels(sigma_e, lambdaL=None) -> np.ndarray:
    """idxS of pre_define_structure_params.m:6-14 (1-based, column-major)."""
    nz = np.abs(np.asarray(sigma_e).ravel(order="F")) > 1e-12
    if lambdaL is not None:
        nz |= np.abs(np.asarray(lambdaL).ravel(order="F")) > 1e-12
    return (np.flatnonzero(nz) + 1).astype(np.int64)


def panel_ids(idxS, L, M, N):
    """lse_generate_panelIDs -> (all_panels_ids (nv, 6) 1-based, num_nodes)."""
    lib = _lib.load()
    idx = np.ascontiguousarray(idxS, dtype=np.int64)
    nv = idx.size
    ap = np.zeros(6 * nv, dtype=np.int64)
    nn = C.c_int64()
    _lib.check(lib.vh_panel_ids(L, M, N, nv, _lib.i64ptr(idx), _lib.i64ptr(ap), C.byref(nn)))
    return ap.reshape(6, nv).T.copy(), nn.value


def incidence(all_panels_ids, num_nodes) -> sp.csc_matrix:
    """lse_compute_Ae_matrix -> Ae (num_nodes x 5 nv), CSC."""
    lib = _lib.load()
    nv = all_panels_ids.shape[0]
    ap = np.ascontiguousarray(all_panels_ids.T.ravel(), dtype=np.int64)
    jc = np.zeros(5 * nv + 1, dtype=np.int64)
    ir = np.zeros(16 * nv, dtype=np.int64)
    pr = np.zeros(16 * nv)
    _lib.check(lib.vh_incidence(nv, _lib.i64ptr(ap), _lib.i64ptr(jc), _lib.i64ptr(ir), _lib.dptr(pr)))
    return sp.csc_matrix((pr, ir, jc), shape=(num_nodes, 5 * nv))


def setup_device(ctx, idxS, L, M, N, with_incidence=True):
    """Panel ids, num_nodes and (optionally) Ae built on the context's device (vh_setup_device):
    the same numbers as panel_ids() and incidence()."""
    lib = _lib.load()
    idx = np.ascontiguousarray(idxS, dtype=np.int64)
    nv = idx.size
    ap = np.zeros(6 * nv, dtype=np.int64)
    nn = C.c_int64()
    if with_incidence:
        jc = np.zeros(5 * nv + 1, dtype=np.int64)
        ir = np.zeros(16 * nv, dtype=np.int64)
        pr = np.zeros(16 * nv)
        bufs = (_lib.i64ptr(jc), _lib.i64ptr(ir), _lib.dptr(pr))
    else:
        bufs = (None, None, None)
    _lib.check(lib.vh_setup_device(ctx.handle, L, M, N, nv, _lib.i64ptr(idx), _lib.i64ptr(ap), C.byref(nn),
                                   *bufs), ctx.handle)
    apid = ap.reshape(6, nv).T.copy()
    if not with_incidence:
        return apid, nn.value, None
    return apid, nn.value, sp.csc_matrix((pr, ir, jc), shape=(nn.value, 5 * nv))


def _node_ids(idxS, shape, apid, rows):
    L, M, N = shape
    rows = np.asarray(rows, dtype=np.int64).reshape(-1, 4)
    lin = (rows[:, 0] - 1) + L * ((rows[:, 1] - 1) + M * (rows[:, 2] - 1)) + 1
    pos = np.searchsorted(idxS, lin)
    ok = (pos < idxS.size) & (idxS[np.minimum(pos, idxS.size - 1)] == lin)
    if not np.all(ok):
        raise ValueError(f"port node on an empty voxel: {rows[~ok][0, :3]}")
    return apid[pos, rows[:, 3] - 1]


def smooth7(n: int) -> int:
    """The least m >= n whose only prime factors are 2, 3, 5 and 7 (lengths the device FFT takes)."""
    m = max(1, int(n))
    while True:
        r = m
        for p in (2, 3, 5, 7):
            while r % p == 0:
                r //= p
        if r == 1:
            return m
        m += 1


def build_problem(sigma_e, lambdaL, dx, pnt_lft, pnt_rght, pnt_well_cond=None, tensor=None, meta=None, ctx=None):
    """Inputs of the solve loop.  tensor: (fN_all2, st2) host arrays, or None to leave the tensor to
    the device (Problem.fN_all2 = None; Sweep then generates it in place).  ctx: a vie.Context to
    number the panels and build Ae on its device (vh_setup_device), else the host builders.

    With the tensor left to the device, a grid whose padded FFT lengths 2L, 2M, 2N have a prime factor
    above 7 is extended with empty voxels at its high ends to the next lengths that do not: the
    operator on the voxels, their order, the panel numbering and the port rows are unchanged (MATLAB's
    FFTW takes any length; the device FFT takes radices 2, 3, 5, 7)."""
    sigma_e = np.asfortranarray(sigma_e)
    L, M, N = sigma_e.shape
    if tensor is None and (smooth7(L), smooth7(M), smooth7(N)) != (L, M, N):
        shape = (smooth7(L), smooth7(M), smooth7(N))
        grown = np.zeros(shape, order="F")
        grown[:L, :M, :N] = sigma_e
        if lambdaL is not None:
            lam = np.zeros(shape, order="F")
            lam[:L, :M, :N] = lambdaL
            lambdaL = lam
        meta = dict(meta or {}, grid_padded_from=(L, M, N))
        sigma_e = grown
        L, M, N = shape
    idxS = nonempty_voxels(sigma_e, lambdaL)
    if ctx is not None:
        apid, num_nodes, Ae = setup_device(ctx, idxS, L, M, N)
    else:
        apid, num_nodes = panel_ids(idxS, L, M, N)
        Ae = incidence(apid, num_nodes)
    nc = Ae.shape[1]
    P = len(pnt_lft)
    rhs = np.zeros((num_nodes + nc, P))
    Aer = Ae.tocsr()
    inj_all, grd_all = [], []
    for p in range(P):
        inj = _node_ids(idxS, (L, M, N), apid, pnt_lft[p]) if len(pnt_lft[p]) else np.zeros(0, np.int64)
        grd = _node_ids(idxS, (L, M, N), apid, pnt_rght[p]) if len(pnt_rght[p]) else np.zeros(0, np.int64)
        if p == 0 and pnt_well_cond is not None and len(pnt_well_cond):
            grd = np.concatenate([grd, _node_ids(idxS, (L, M, N), apid, pnt_well_cond)])
        rhs[:nc, p] = -np.asarray(Aer[inj - 1, :].sum(axis=0)).ravel()
        inj_all.append(inj)
        grd_all.append(grd)
    inj = np.concatenate(inj_all) if inj_all else np.zeros(0, np.int64)
    grd = np.concatenate(grd_all) if grd_all else np.zeros(0, np.int64)
    keep = np.ones(num_nodes, dtype=bool)
    keep[grd - 1] = False
    keep[inj - 1] = False
    rhs = rhs[: rhs.shape[0] - grd.size - inj.size]
    Ar = Aer[keep, :]
    Ar = Ar[np.diff(Ar.indptr) > 0, :].tocsc()
    Ar.sort_indices()
    fN, st = (None, None) if tensor is None else tensor
    m = dict(meta or {})
    m.update(nodeid_4_grnd=grd, nodeid_4_injectcurr=inj, num_nodes=num_nodes)
    return Problem(L, M, N, float(dx), sigma_e, lambdaL, idxS, Ar, rhs, fN, st, meta=m)


def problem_from_workload(w, tensor=None, ctx=None) -> Problem:
    return build_problem(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght, tensor=tensor,
                         meta={"name": w.name}, ctx=ctx)


def circulant_tensor(L, M, N, dx, ctx=None):
    """lse_generate_circulant_tensor(dx, 1, L, M, N, 0) on the device -> (fN_all2, st2) host arrays."""
    from . import vie

    ctx = ctx or vie.default_context()
    fN = np.zeros(7 * 8 * L * M * N, dtype=np.complex128)
    st = np.zeros(3, dtype=np.complex128)
    _lib.check(ctx._lib.vh_circulant_tensor(ctx.handle, L, M, N, float(dx), _lib.cview(fN), _lib.cview(st)), ctx.handle)
    return fN.reshape((2 * L, 2 * M, 2 * N, 7), order="F"), st
