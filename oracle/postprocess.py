"""Oracle: current post-processing of the reference (test infrastructure).

Restates src_post_process/post_obtain_curr_coefs_on_grid.m:1-45 and
src_post_process/post_obtain_currs_on_nodes.m:1-196 (no plotting).  MATLAB conventions:
column-major grids, `find` returns the entries of a sparse matrix column by column.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

TOLA = 1e-12   # post_obtain_curr_coefs_on_grid.m:5, post_obtain_currs_on_nodes.m:15


def post_obtain_curr_coefs_on_grid(x, Mc):
    """-> (Jx, Jy, Jz, J2d, J3d) on the (L, M, N) grid, cmin, cmax (post_obtain_curr_coefs_on_grid.m)."""
    L, M, N = Mc.shape
    ignore = np.abs(np.asarray(Mc).ravel(order="F")) < TOLA          # :8-18
    nn = int((~ignore).sum())                                        # :20-21
    parts = [np.asarray(x)[k * nn:(k + 1) * nn] for k in range(5)]   # :23-24
    absj = np.abs(np.concatenate(parts[:3]))
    cmin, cmax = absj.min(), absj.max()                              # :26-27
    grids = []
    for p in parts:                                                   # :32-45
        g = np.zeros(L * M * N, dtype=np.result_type(p, np.float64))
        g[~ignore] = p
        grids.append(g.reshape((L, M, N), order="F"))
    return (*grids, cmin, cmax)


def _find(A):
    """MATLAB [rows, cols] = find(A) for a sparse matrix: column by column, rows ascending (0-based)."""
    A = sp.csc_matrix(A)
    A.eliminate_zeros()
    A.sort_indices()
    cols = np.repeat(np.arange(A.shape[1]), np.diff(A.indptr))
    return A.indices.astype(np.int64), cols


def post_obtain_currs_on_nodes(x, Ae_only_leaving, Ae_only_entering_bndry, r, Mc, dx):
    """-> (nodes_w_currs_x_aligned, ..._y_aligned, ..._z_aligned), rows [x y z current]
    (post_obtain_currs_on_nodes.m)."""
    num_curr = Ae_only_leaving.shape[1]
    nv = num_curr // 5
    xj = np.asarray(x)[:num_curr]
    x_node = -(Ae_only_leaving @ xj) + Ae_only_entering_bndry @ xj                       # :7-10
    L, M, N = Mc.shape
    keep = np.abs(np.asarray(Mc).ravel(order="F")) > TOLA                               # :16-30
    cens = np.asarray(r).reshape(L * M * N, 3, order="F")[keep]
    voxc = np.vstack([cens, cens, cens])
    trunc = sp.diags((np.arange(num_curr) < 3 * nv).astype(np.float64))                   # :35-38
    A1 = sp.csc_matrix(Ae_only_leaving) @ trunc
    A2 = sp.csc_matrix(Ae_only_entering_bndry) @ trunc
    rows, cols = _find(A1)                                                                # :40-41
    rows2, cols2 = _find(A2)

    def positions(cs, sign):                                                              # :48-62, :71-87
        pos = voxc[cs].copy()
        axis = np.minimum(cs // nv, 2)
        pos[np.arange(len(cs)), axis] += sign * dx / 2
        return pos

    nodes = np.zeros((len(rows) + len(rows2), 5), dtype=np.complex128)
    nodes[: len(rows), :3] = positions(cols, -1)
    nodes[: len(rows), 3] = x_node[rows]
    nodes[: len(rows), 4] = rows + 1
    nodes[len(rows):, :3] = positions(cols2, +1)
    nodes[len(rows):, 3] = x_node[rows2]
    nodes[len(rows):, 4] = rows2 + 1
    ids = np.concatenate([rows, rows2])
    size = max(len(ids), int(ids.max()) + 1 if len(ids) else 0)                           # :102-105
    srt = np.zeros((size, 4), dtype=np.complex128)
    last = {}
    for k, i in enumerate(ids):   # repeated node ids: the last assignment wins
        last[int(i)] = k
    sel = np.array(sorted(last.items()), dtype=np.int64).reshape(-1, 2)
    srt[sel[:, 0]] = nodes[sel[:, 1], :4]

    out = []
    for c in range(3):                                                                    # :110-196
        t = np.zeros(num_curr)
        t[c * nv:(c + 1) * nv] = 1.0
        ex = np.flatnonzero(A1 @ t)
        en = np.flatnonzero(A2 @ t)
        out.append(srt[np.concatenate([ex, en])])
    return tuple(out)
