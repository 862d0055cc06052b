"""Post-processing of the solution currents (src_post_process of the reference), without plotting.

post_obtain_curr_coefs_on_grid(x, Mc)   post_obtain_curr_coefs_on_grid.m:1-45: the five current
    coefficients of each voxel scattered onto (L, M, N) grids -- on the device (vh_currents_on_grid).
post_obtain_currs_on_nodes(x, Ae_only_leaving, Ae_only_entering_bndry, r, Mc, dx)
    post_obtain_currs_on_nodes.m:1-196: the currents on the panel nodes, -Ae_only_leaving x +
    Ae_only_entering_bndry x (one device product with the difference matrix, vh_sparse_matvec),
    placed half a voxel from the voxel centres `r` along the panel's axis and sorted into x-, y- and
    z-aligned node lists with rows [x y z current].
Both take one solution (n,) or a batch (B, n); the batch form returns one result per row.
incidence_split(all_panels_ids, num_nodes) gives Ae_only_leaving and Ae_only_entering_bndry from the
panel ids (lse_compute_Ae_matrix.m:94-113) for callers without them.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import _lib, vie

TOLA = 1e-12


def _batch(x):
    x = np.asarray(x)
    return (x[None, :] if x.ndim == 1 else x), x.ndim == 1


def post_obtain_curr_coefs_on_grid(x, Mc, ctx: vie.Context | None = None):
    """-> (Jx, Jy, Jz, J2d, J3d, cmin, cmax); each J a complex (L, M, N) grid (a (B, L, M, N) stack
    for a batch), cmin / cmax the extreme |Jx|, |Jy|, |Jz| (arrays of B for a batch)."""
    ctx = ctx or vie.default_context()
    X, single = _batch(x)
    L, M, N = np.shape(Mc)
    idxS = np.flatnonzero(np.abs(np.asarray(Mc).ravel(order="F")) >= TOLA).astype(np.int64) + 1
    nv = idxS.size
    B = X.shape[0]
    Xc = np.ascontiguousarray(X.astype(np.complex128))
    grids = np.empty((B, 5, L * M * N), dtype=np.complex128)
    _lib.check(ctx._lib.vh_currents_on_grid(ctx.handle, L, M, N, nv, _lib.i64ptr(idxS), B, _lib.cview(Xc),
                                            Xc.shape[1], _lib.cview(grids)), ctx.handle)
    absj = np.abs(Xc[:, : 3 * nv])
    cmin, cmax = absj.min(axis=1), absj.max(axis=1)
    g = grids.reshape(B, 5, N, M, L).transpose(0, 1, 4, 3, 2)   # column-major (L, M, N) per component
    if single:
        return (*[g[0, c] for c in range(5)], cmin[0], cmax[0])
    return (*[g[:, c] for c in range(5)], cmin, cmax)


def incidence_split(all_panels_ids, num_nodes):
    """(Ae, Ae_only_leaving, Ae_only_entering_bndry) from the panel ids (lse_compute_Ae_matrix.m:29-113):
    the leaving part keeps the entries of the minus-side panels (-x, -y, -z); the entering part keeps
    the rows of the nodes into which only current from Jx, Jy, Jz enters (row sum over them == +1)."""
    from . import structure

    apid = np.asarray(all_panels_ids, dtype=np.int64)
    nv = apid.shape[0]
    Ae = structure.incidence(apid, num_nodes).tocsc()
    Ae.sort_indices()
    row = Ae.indices
    col = np.repeat(np.arange(Ae.shape[1]), np.diff(Ae.indptr))
    v = col % nv
    # the panel of each entry: its row is the node id of one of the voxel's six panels
    pan = np.full(row.shape, -1)
    for p in range(6):
        pan = np.where(apid[v, p] - 1 == row, p, pan)
    leave = np.isin(pan, (0, 2, 4))
    Ae_leave = sp.csc_matrix((Ae.data[leave], (row[leave], col[leave])), shape=Ae.shape)
    jsum = np.asarray(Ae[:, : 3 * nv].sum(axis=1)).ravel()
    enter_rows = np.abs(jsum - 1.0) == 0.0
    keep = enter_rows[row]
    Ae_enter = sp.csc_matrix((Ae.data[keep], (row[keep], col[keep])), shape=Ae.shape)
    return Ae, Ae_leave, Ae_enter


def post_obtain_currs_on_nodes(x, Ae_only_leaving, Ae_only_entering_bndry, r, Mc, dx,
                               ctx: vie.Context | None = None):
    """-> (nodes_w_currs_x_aligned, nodes_w_currs_y_aligned, nodes_w_currs_z_aligned), rows [x y z current]
    (a list of such triples for a batch)."""
    ctx = ctx or vie.default_context()
    X, single = _batch(x)
    B = X.shape[0]
    A1 = sp.csc_matrix(Ae_only_leaving)
    A2 = sp.csc_matrix(Ae_only_entering_bndry)
    num_nodes, num_curr = A1.shape
    nv = num_curr // 5
    D = (A2 - A1).tocsc()
    D.sort_indices()
    jc = np.ascontiguousarray(D.indptr, dtype=np.int64)
    ir = np.ascontiguousarray(D.indices, dtype=np.int64)
    pr = np.ascontiguousarray(D.data, dtype=np.float64)
    Xc = np.ascontiguousarray(X.astype(np.complex128))
    xnode = np.empty((B, num_nodes), dtype=np.complex128)
    _lib.check(ctx._lib.vh_sparse_matvec(ctx.handle, num_nodes, num_curr, _lib.i64ptr(jc), _lib.i64ptr(ir),
                                         _lib.dptr(pr), B, _lib.cview(Xc), Xc.shape[1], _lib.cview(xnode),
                                         num_nodes), ctx.handle)
    L, M, N = np.shape(Mc)
    keep = np.abs(np.asarray(Mc).ravel(order="F")) > TOLA
    cens = np.asarray(r, dtype=np.float64).reshape(L * M * N, 3, order="F")[keep]
    voxc = np.concatenate([cens, cens, cens])
    # the Jx, Jy, Jz columns of both matrices, entries column by column (MATLAB find order)
    entries = []
    for A, sign in ((A1, -1.0), (A2, +1.0)):
        T = A[:, : 3 * nv].tocsc()
        T.eliminate_zeros()
        T.sort_indices()
        cols = np.repeat(np.arange(T.shape[1]), np.diff(T.indptr))
        entries.append((T, T.indices.astype(np.int64), cols, sign))
    ids = np.concatenate([e[1] for e in entries])
    pos = np.concatenate([voxc[e[2]] for e in entries])
    axis = np.concatenate([np.minimum(e[2] // nv, 2) for e in entries])
    shift = np.concatenate([np.full(len(e[2]), e[3]) for e in entries])
    pos[np.arange(len(ids)), axis] += shift * dx / 2
    # node table indexed by node id; for a node listed twice the later row counts
    size = max(len(ids), int(ids.max()) + 1 if len(ids) else 0)
    last = np.full(size, -1, dtype=np.int64)
    uid, first_in_reversed = np.unique(ids[::-1], return_index=True)
    last[uid] = len(ids) - 1 - first_in_reversed   # the last listing of each node id
    have = np.flatnonzero(last >= 0)
    aligned_rows = []
    for c in range(3):
        t = np.zeros(num_curr)
        t[c * nv:(c + 1) * nv] = 1.0
        ex = np.flatnonzero(entries[0][0] @ t[: 3 * nv])
        en = np.flatnonzero(entries[1][0] @ t[: 3 * nv])
        aligned_rows.append(np.concatenate([ex, en]))
    results = []
    for b in range(B):
        srt = np.zeros((size, 4), dtype=np.complex128)
        srt[have, :3] = pos[last[have]]
        srt[have, 3] = xnode[b, ids[last[have]]]
        results.append(tuple(srt[rows] for rows in aligned_rows))
    return results[0] if single else results
