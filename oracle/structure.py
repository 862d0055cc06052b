"""Oracle: panel numbering, incidence matrix Ae, port nodes and RHS (test infrastructure).

Restates, in vectorised NumPy:
  * src_lse_formation/lse_generate_panelIDs.m:1-176  (panel numbering)
  * src_lse_formation/lse_compute_Ae_matrix.m:1-113   (Ae, Ae_only_leaving, Ae_only_entering_bndry)
  * src_lse_formation/lse_assign_exc_grnd_nodes.m:1-94 (port node ids)
  * VoxHenry_executer.m:159-193                         (RHS, removal of port rows -> Ar)
Panel/node ids are 1-based, as in the reference.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp


def _panels_along(occ: np.ndarray, perm: tuple[int, int, int]) -> tuple[np.ndarray, np.ndarray, int]:
    """Number the panels along one axis.

    ``occ`` is the (L, M, N) voxel occupancy; ``perm`` lists the axes from the
    scan's fastest to slowest index (the scanned axis first).  Returns the
    left/right panel ids (1-based, per voxel in the scan order), the voxel
    linear indices (Fortran) in scan order and the number of panels.
    lse_generate_panelIDs.m:35-67 (x), :78-113 (y), :122-157 (z): every
    non-empty voxel takes ids (k, k+1); k advances by one more when the next
    voxel along the scanned axis is empty or outside the grid.
    """
    shape = occ.shape
    lin = np.arange(occ.size).reshape(shape, order="F")
    # arrange so the scanned axis is fastest: transpose to (fast, mid, slow) then Fortran-ravel
    occ_t = np.transpose(occ, perm)
    lin_t = np.transpose(lin, perm)
    flat_occ = occ_t.ravel(order="F")
    flat_lin = lin_t.ravel(order="F")
    # "next voxel along the scanned axis is non-empty"
    nxt = np.zeros_like(occ_t)
    nxt[:-1] = occ_t[1:]
    flat_next = nxt.ravel(order="F")
    sel = flat_occ
    vox_lin = flat_lin[sel]
    run_end = ~flat_next[sel]
    nv = vox_lin.size
    left = np.arange(nv, dtype=np.int64) + 1
    # exclusive cumulative count of run ends before each voxel
    ends_before = np.concatenate([[0], np.cumsum(run_end)[:-1]]).astype(np.int64)
    left = left + ends_before
    right = left + 1
    npanels = int(right.max()) if nv else 0
    return left, right, vox_lin, npanels


def generate_panel_ids(idxS: np.ndarray, L: int, M: int, N: int):
    """lse_generate_panelIDs.m: returns (all_panels_ids (Nv, 6) int64 1-based, num_nodes)."""
    nv = idxS.size
    flat = np.zeros(L * M * N, dtype=bool)
    flat[idxS - 1] = True
    occ = flat.reshape((L, M, N), order="F")
    vnum = np.zeros(L * M * N, dtype=np.int64)
    vnum[idxS - 1] = np.arange(nv)          # boolean_tens (0-based voxel number)
    out = np.zeros((nv, 6), dtype=np.int64)
    # x panels: scan x (fast), y, z (slow)
    lx, rx, vl, npx = _panels_along(occ, (0, 1, 2))
    out[vnum[vl], 0], out[vnum[vl], 1] = lx, rx
    # y panels: scan y (fast), z, x (slow)   (loops ll / nn / mm, lse_generate_panelIDs.m:78-80)
    ly, ry, vl, npy = _panels_along(occ, (1, 2, 0))
    out[vnum[vl], 2], out[vnum[vl], 3] = ly + npx, ry + npx
    # z panels: scan z (fast), x, y (slow)   (loops mm / ll / nn, lse_generate_panelIDs.m:122-124)
    lz, rz, vl, npz = _panels_along(occ, (2, 0, 1))
    out[vnum[vl], 4], out[vnum[vl], 5] = lz + npx + npy, rz + npx + npy
    return out, npx + npy + npz


# Per-voxel incidence coefficients: column block c (Jx, Jy, Jz, J2D, J3D) x local panel
# (-x, +x, -y, +y, -z, +z).  lse_compute_Ae_matrix.m:205-262.
AE_LOCAL = np.array(
    [
        [-1.0, 1.0, 0.0, 0.0, 0.0, 0.0],     # Jx
        [0.0, 0.0, -1.0, 1.0, 0.0, 0.0],     # Jy
        [0.0, 0.0, 0.0, 0.0, -1.0, 1.0],     # Jz
        [0.5, 0.5, -0.5, -0.5, 0.0, 0.0],    # J2D (Jfx +1/2, Jfy -1/2)
        [0.5, 0.5, 0.5, 0.5, -1.0, -1.0],    # J3D (Jsx, Jsy +1/2, Jsz -1)
    ]
)


def compute_Ae(all_panels_ids: np.ndarray, num_nodes: int):
    """lse_compute_Ae_matrix.m:29-113 -> (Ae, Ae_only_leaving, Ae_only_entering_bndry), CSC."""
    nv = all_panels_ids.shape[0]
    rows, cols, vals = [], [], []
    lrows, lcols, lvals = [], [], []
    kk = np.arange(nv)
    for c in range(5):
        for p in range(6):
            v = AE_LOCAL[c, p]
            if v == 0.0:
                continue
            rows.append(all_panels_ids[:, p] - 1)
            cols.append(kk + c * nv)
            vals.append(np.full(nv, v))
            # "only leaving" keeps the minus-side panel (-x, -y, -z) entries:
            # lse_compute_Ae_matrix.m:213-215, 223, 232, 242, 251, 260
            if p in (0, 2, 4):
                lrows.append(all_panels_ids[:, p] - 1)
                lcols.append(kk + c * nv)
                lvals.append(np.full(nv, v))
    shape = (num_nodes, 5 * nv)
    Ae = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=shape)
    Ae.sort_indices()
    Ae_leave = sp.csc_matrix((np.concatenate(lvals), (np.concatenate(lrows), np.concatenate(lcols))), shape=shape)
    Ae_leave.sort_indices()
    # nodes where current only enters (boundary): Ae * [1 (Jx,Jy,Jz); 0] == +1
    dum = np.zeros(5 * nv)
    dum[: 3 * nv] = 1.0
    res = Ae @ dum
    enter = np.flatnonzero(res == 1)
    mask = np.zeros(num_nodes, dtype=bool)
    mask[enter] = True
    coo = Ae.tocoo()
    keep = mask[coo.row]
    Ae_enter = sp.csc_matrix((coo.data[keep], (coo.row[keep], coo.col[keep])), shape=shape)
    Ae_enter.sort_indices()
    return Ae, Ae_leave, Ae_enter


def _lookup_voxel(idxS: np.ndarray, shape, pts: np.ndarray) -> np.ndarray:
    """sub2ind + lookup in idxS (lse_assign_exc_grnd_nodes.m:14-26) -> 0-based voxel numbers."""
    L, M, N = shape
    lin = (pts[:, 0] - 1) + L * ((pts[:, 1] - 1) + M * (pts[:, 2] - 1)) + 1
    pos = np.searchsorted(idxS, lin)
    ok = (pos < idxS.size) & (idxS[np.minimum(pos, idxS.size - 1)] == lin)
    if not np.all(ok):
        bad = pts[~ok][0]
        raise ValueError(f"cannot find non-empty voxel for port node at voxel {tuple(bad[:3])}")
    return pos


def assign_exc_grnd_nodes(idxS, shape, all_panels_ids, port_no, pnt_lft, pnt_rght, pnt_well_cond):
    """lse_assign_exc_grnd_nodes.m:1-94 (port_no is 1-based). Returns (grnd, inject) node ids, 1-based."""
    lft = pnt_lft[port_no - 1]
    rgt = pnt_rght[port_no - 1]
    inj = all_panels_ids[_lookup_voxel(idxS, shape, lft), lft[:, 3] - 1] if len(lft) else np.zeros(0, np.int64)
    grd = all_panels_ids[_lookup_voxel(idxS, shape, rgt), rgt[:, 3] - 1] if len(rgt) else np.zeros(0, np.int64)
    if pnt_well_cond is not None and len(pnt_well_cond) and port_no == 1:
        w = all_panels_ids[_lookup_voxel(idxS, shape, pnt_well_cond), pnt_well_cond[:, 3] - 1]
        grd = np.concatenate([grd, w])
    return grd.astype(np.int64), inj.astype(np.int64)


@dataclass
class System:
    """Everything the executer builds before the frequency loop (VoxHenry_executer.m:69-200)."""
    L: int
    M: int
    N: int
    dx: float
    sigma_e: np.ndarray
    lambdaL: np.ndarray | None
    idxS: np.ndarray          # 1-based
    idxS5: np.ndarray         # 1-based
    all_panels_ids: np.ndarray
    num_nodes: int
    Ae_full: sp.csc_matrix    # before port-row removal
    Ar: sp.csc_matrix         # port rows removed ("Ae" inside the solve)
    rhs: np.ndarray           # (nc + nphi, num_ports) float64
    nodeid_4_grnd: np.ndarray
    nodeid_4_injectcurr: np.ndarray
    Ae_only_leaving: sp.csc_matrix
    Ae_only_entering_bndry: sp.csc_matrix

    @property
    def nv(self):
        return self.idxS.size

    @property
    def nc(self):
        return 5 * self.idxS.size

    @property
    def nphi(self):
        return self.Ar.shape[0]

    @property
    def n(self):
        return self.nc + self.nphi


def build_system(sigma_e, lambdaL, dx, pnt_lft, pnt_rght, pnt_well_cond=None) -> System:
    from .vhr import structure_params

    L, M, N = sigma_e.shape
    idxS, idxS5 = structure_params(sigma_e, lambdaL)
    apid, num_nodes = generate_panel_ids(idxS, L, M, N)
    Ae, Ae_leave, Ae_enter = compute_Ae(apid, num_nodes)
    nc = Ae.shape[1]
    num_ports = len(pnt_lft)
    rhs = np.zeros((num_nodes + nc, num_ports))
    inj_all, grd_all = [], []
    Aer = Ae.tocsr()
    for p in range(1, num_ports + 1):
        g, i = assign_exc_grnd_nodes(idxS, (L, M, N), apid, p, pnt_lft, pnt_rght, pnt_well_cond)
        inj_all.append(i)
        grd_all.append(g)
        # exc_vect = sum(-Ae(inject,:), 1)   (VoxHenry_executer.m:175-177)
        exc = -np.asarray(Aer[i - 1, :].sum(axis=0)).ravel()
        rhs[:nc, p - 1] = exc
    inj = np.concatenate(inj_all) if inj_all else np.zeros(0, np.int64)
    grd = np.concatenate(grd_all) if grd_all else np.zeros(0, np.int64)
    # VoxHenry_executer.m:181-193: zero port rows, truncate rhs, drop empty rows
    keep = np.ones(num_nodes, dtype=bool)
    keep[grd - 1] = False
    keep[inj - 1] = False
    rhs = rhs[: rhs.shape[0] - grd.size - inj.size, :]
    Ar = Aer[keep, :]
    nz_rows = np.diff(Ar.indptr) > 0
    Ar = Ar[nz_rows, :].tocsc()
    Ar.sort_indices()
    return System(
        L=L, M=M, N=N, dx=dx, sigma_e=sigma_e, lambdaL=lambdaL, idxS=idxS, idxS5=idxS5,
        all_panels_ids=apid, num_nodes=num_nodes, Ae_full=Ae, Ar=Ar, rhs=rhs,
        nodeid_4_grnd=grd, nodeid_4_injectcurr=inj,
        Ae_only_leaving=Ae_leave, Ae_only_entering_bndry=Ae_enter,
    )
