"""Oracle: circulant Green tensor of the VIE operator (test infrastructure).

Restates src_lse_formation/lse_generate_circulant_tensor.m:1-833 for the
default settings of the reference (lse_enhanced_near = 3,
lse_exploit_symmetry = 1, fl_oneoverr_kernel = 1 -> ko_grfn = 1e-30), with
src_lin_vie/cubatures/volume_volume.m:1-117, volume_volume_sym.m:1-121,
weights_points.m:1-99 (Gauss-Legendre tensor rules), fft_operator.m and
gperiodic_coeff_nop_linJVIE.m.

Near-field interactions (offsets 0..1 in every axis) come from the
reference's precomputed table src_lin_vie/K_near_interactions_1mm.txt
(6 rows x 3 complex values for a 1 mm voxel), scaled by (dx/1e-3)^{5,6,7}
(lse_generate_circulant_tensor.m:363-400).  The table is data: its values
are reproduced below.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.fft as sfft

WORKERS = os.cpu_count() or 1   # the host cores (the reference's MATLAB is multithreaded)

# src_lin_vie/K_near_interactions_1mm.txt (rows: offsets (1,1,1),(1,2,1),(1,2,2),(2,1,1),(2,2,1),(2,2,2);
# columns: pulse-pulse, linear(x)-pulse, linear(x)-linear(x') for a 1 mm voxel)
K_NEAR_1MM = np.array(
    [
        [1.497896808995041e-016 - 5.003461427972696e-027j, -1.884273158210909e-037 - 2.012211605895784e-048j, 2.910077873947119e-024 - 3.626541131608855e-051j],
        [7.805636278778824e-017 - 5.003461427972697e-027j, 1.206473223753176e-035 - 4.160008679876429e-049j, 6.11217610670709e-025 - 2.004923164762494e-052j],
        [5.638025079837469e-017 - 5.003461427972694e-027j, 2.412452305035321e-035 + 2.98904327368899e-049j, 2.297463434675418e-025 - 5.006665539022287e-052j],
        [7.805636278778813e-017 - 5.003461427972696e-027j, -5.757414693177654e-021 - 7.50496380728818e-048j, -7.440943011730615e-025 - 1.219881017509337e-051j],
        [5.638025079837419e-017 - 5.003461427972694e-027j, -2.390823543614732e-021 - 3.06145823959795e-048j, -1.275734678285788e-025 + 1.681050961223937e-051j],
        [4.605920193990263e-017 - 5.003461427972694e-027j, -1.321546896796384e-021 + 2.534523806813602e-049j, -1.402863426594222e-026 - 1.963545763613549e-051j],
    ],
    dtype=np.complex128,
)

# gperiodic_coeff_nop_linJVIE.m: sign of each of the 7 components when mirrored across
# the listed axes (cube 'L' = x, 'M' = y, 'N' = z).
GP_COEFF = {
    "L": np.array([+1, -1, +1, +1, +1, +1, +1], dtype=np.float64),
    "M": np.array([+1, +1, -1, +1, +1, +1, +1], dtype=np.float64),
    "N": np.array([+1, +1, +1, +1, -1, +1, +1], dtype=np.float64),
    "LM": np.array([+1, -1, -1, +1, +1, +1, +1], dtype=np.float64),
    "LN": np.array([+1, -1, +1, +1, -1, +1, +1], dtype=np.float64),
    "MN": np.array([+1, +1, -1, +1, -1, +1, +1], dtype=np.float64),
    "LMN": np.array([+1, -1, -1, +1, -1, +1, +1], dtype=np.float64),
}

KO_GRFN = 1e-30   # lse_generate_circulant_tensor.m:21-23


def weights_points(n: int, dim: int = 6):
    """weights_points.m: tensor Gauss-Legendre rule on [-1, 1]^dim -> (W, [X, Y, Z, Xp, Yp, Zp])."""
    x1, w1 = np.polynomial.legendre.leggauss(n)
    grids = np.meshgrid(*([x1] * dim), indexing="ij")
    wg = np.meshgrid(*([w1] * dim), indexing="ij")
    W = np.ones(n**dim)
    for g in wg:
        W = W * g.ravel(order="F")
    pts = [g.ravel(order="F") for g in grids]
    return W, pts


def _kernel_far(R, k0):
    # volume_volume.m:25 (volume_ker = 1): 1/4/pi * exp(-1j*k0*R) ./ R
    return (1 / 4 / np.pi) * np.exp(-1j * k0 * R) / R


def volume_volume_batch(W, pts, k0, r_m, dx):
    """volume_volume.m (volume_ker = 1) for a batch of observation centres r_m (C, 3) and r_n = 0.

    Returns I (C, 7): Gxx, G2D,x, G2D,y, G2D,2D, G3D,z, G2D,3D, G3D,3D.
    """
    X, Y, Z, Xp, Yp, Zp = pts
    J = (dx / 2) ** 6
    h = dx / 2
    Xg = r_m[:, 0:1] + h * X[None, :]
    Yg = r_m[:, 1:2] + h * Y[None, :]
    Zg = r_m[:, 2:3] + h * Z[None, :]
    R = np.sqrt((Xg - h * Xp[None, :]) ** 2 + (Yg - h * Yp[None, :]) ** 2 + (Zg - h * Zp[None, :]) ** 2)
    Xt, Yt, Zt = h * X, h * Y, h * Z
    Xpb, Ypb, Zpb = h * Xp, h * Yp, h * Zp
    # a centre at the origin (the self cell) has coincident points (R = 0): its entries are not
    # finite here and are replaced by the near-field values afterwards
    with np.errstate(divide="ignore", invalid="ignore"):
        ker = _kernel_far(R, k0)
        Wk = W[None, :] * ker
        K1 = Wk.sum(axis=1) * J
        K3 = (Wk * Xt[None, :]).sum(axis=1) * J
        K5 = (Wk * Yt[None, :]).sum(axis=1) * J
        K7 = (Wk * Zt[None, :]).sum(axis=1) * J
        K8 = (Wk * (Xpb * Xt)[None, :]).sum(axis=1) * J
        K9 = (Wk * (Ypb * Yt)[None, :]).sum(axis=1) * J
        K10 = (Wk * (Zpb * Zt)[None, :]).sum(axis=1) * J
    # volume_volume.m:100-115
    return np.stack([K1, -K3, K5, K8 + K9, 2 * K7, K8 - K9, K8 + K9 + 4 * K10], axis=1)


def volume_volume_sym_batch(W, pts, k0, r_m, dx):
    """volume_volume_sym.m (dir = 1, volume_ker = 1) -> (C, 3): pulse-pulse, lin(x)-pulse, lin(x)-lin(x')."""
    X, Y, Z, Xp, Yp, Zp = pts
    J = (dx / 2) ** 6
    h = dx / 2
    Xg = r_m[:, 0:1] + h * X[None, :]
    Yg = r_m[:, 1:2] + h * Y[None, :]
    Zg = r_m[:, 2:3] + h * Z[None, :]
    R = np.sqrt((Xg - h * Xp[None, :]) ** 2 + (Yg - h * Yp[None, :]) ** 2 + (Zg - h * Zp[None, :]) ** 2)
    # the self cell's coincident points (R = 0) give non-finite entries, replaced by the near-field
    # values afterwards
    with np.errstate(divide="ignore", invalid="ignore"):
        ker = _kernel_far(R, k0)
        Wk = W[None, :] * ker
        K1 = Wk.sum(axis=1) * J
        K2 = (Wk * (h * X)[None, :]).sum(axis=1) * J
        K3 = (Wk * ((h * Xp) * (h * X))[None, :]).sum(axis=1) * J
    return np.stack([K1, K2, K3], axis=1)


def _sym_index_list(nL: int, nM: int, nN: int):
    """inter_idx of lse_generate_circulant_tensor.m:151-161 / :342-352 as 1-based (mx, my, mz)."""
    out = []
    for mx in range(1, nL + 1):
        for my in range(1, nM + 1):
            for mz in range(1, my + 1):
                out.append((mx, my, mz))
    return out


def _scatter_sym(G, idx, K):
    """Symmetric fill of G from x-direction integrals (lse_generate_circulant_tensor.m:184-305, 405-490)."""
    with np.errstate(invalid="ignore"):
        for (mx, my, mz), (k1, k2, k3) in zip(idx, K):
            a, b, c = mx - 1, my - 1, mz - 1
            G[a, b, c, 0] = k1
            G[a, b, c, 1] = -k2
            G[a, b, c, 3] += k3
            G[a, b, c, 5] += k3
            G[a, b, c, 6] += k3
            if my != mz:
                G[a, c, b, 0] = k1
                G[a, c, b, 1] = -k2
                G[a, c, b, 3] += k3
                G[a, c, b, 5] += k3
                G[a, c, b, 6] += k3
            G[c, a, b, 2] = k2
            G[c, a, b, 3] += k3
            G[c, a, b, 5] -= k3
            G[c, a, b, 6] += k3
            if my != mz:
                G[b, a, c, 2] = k2
                G[b, a, c, 3] += k3
                G[b, a, c, 5] -= k3
                G[b, a, c, 6] += k3
            G[b, c, a, 4] = 2 * k2
            G[b, c, a, 6] += 4 * k3
            if my != mz:
                G[c, b, a, 4] = 2 * k2
                G[c, b, a, 6] += 4 * k3


def green_tensor(dx: float, L: int, M: int, N: int, ko: float = 1.0, chunk: int = 2048):
    """G_mn (L, M, N, 7) complex128 and st_sparse_precon (3,), lse_generate_circulant_tensor.m:52-772."""
    if min(L, M, N) < 2:
        raise NotImplementedError("grids thinner than 2 voxels need the DIRECTFN singular-integral path")
    G = np.zeros((L, M, N, 7), dtype=np.complex128, order="F")
    # far interactions, 3^6 Gauss-Legendre (:56-74)
    W, pts = weights_points(3, 6)
    mx, my, mz = np.meshgrid(np.arange(L), np.arange(M), np.arange(N), indexing="ij")
    offs = np.stack([mx.ravel(order="F"), my.ravel(order="F"), mz.ravel(order="F")], axis=1)
    flat = G.reshape(L * M * N, 7, order="F")

    def far_chunk(s):   # numpy releases the GIL inside the array operations: chunks run on all cores
        flat[s:s + chunk] = volume_volume_batch(W, pts, KO_GRFN, offs[s:s + chunk] * dx, dx)

    with ThreadPoolExecutor(max_workers=WORKERS) as ex:
        list(ex.map(far_chunk, range(0, offs.shape[0], chunk)))
    G = flat.reshape(L, M, N, 7, order="F")
    # medium interactions, 5^6 Gauss-Legendre (:79-310)
    W5, pts5 = weights_points(5, 6)
    nL, nM, nN = min(5, L), min(5, M), min(5, N)
    if nL != nM or nL != nN:
        mxm, mym, mzm = np.meshgrid(np.arange(nL), np.arange(nM), np.arange(nN), indexing="ij")
        o = np.stack([mxm.ravel(order="F"), mym.ravel(order="F"), mzm.ravel(order="F")], axis=1)
        vals = volume_volume_batch(W5, pts5, KO_GRFN, o * dx, dx)
        for (a, b, c), v in zip(o, vals):
            G[a, b, c, :] = v
    else:
        idx = _sym_index_list(nL, nM, nN)
        r_m = (np.array(idx, dtype=np.float64) - 1) * dx
        Ktmp = volume_volume_sym_batch(W5, pts5, KO_GRFN, r_m, dx)
        G[:nL, :nM, :nN, :] = 0
        _scatter_sym(G, idx, Ktmp)
    # near interactions from the precomputed table (:328-492)
    Ls, Ms, Ns = min(2, L), min(2, M), min(2, N)
    idx = _sym_index_list(Ls, Ms, Ns)
    Kn = K_NEAR_1MM.copy()
    s = dx / 1e-3
    Kn[:, 0] *= s**5
    Kn[:, 1] *= s**6
    Kn[:, 2] *= s**7
    G[:Ls, :Ms, :Ns, :] = 0
    _scatter_sym(G, idx, Kn)
    # normalisation (:761-768)
    G = G / dx**4 * ko**2
    G[..., 1:3] *= 1 / dx
    G[..., 3] *= 1 / dx**2
    G[..., 4] *= 1 / dx
    G[..., 5:7] *= 1 / dx**2
    st = np.array([G[0, 0, 0, 0], G[0, 0, 0, 3], G[0, 0, 0, 6]])
    return G, st


def circulant_embed(G: np.ndarray) -> np.ndarray:
    """Gp (2L, 2M, 2N, 7): lse_generate_circulant_tensor.m:776-816."""
    L, M, N, _ = G.shape
    Gp = np.zeros((2 * L, 2 * M, 2 * N, 7), dtype=G.dtype, order="F")
    Gp[:L, :M, :N] = G
    rL, rM, rN = slice(L - 1, 0, -1), slice(M - 1, 0, -1), slice(N - 1, 0, -1)
    c = GP_COEFF
    Gp[L + 1:, :M, :N] = G[rL, :M, :N] * c["L"]
    Gp[:L, M + 1:, :N] = G[:L, rM, :N] * c["M"]
    Gp[:L, :M, N + 1:] = G[:L, :M, rN] * c["N"]
    Gp[L + 1:, M + 1:, :N] = G[rL, rM, :N] * c["LM"]
    Gp[L + 1:, :M, N + 1:] = G[rL, :M, rN] * c["LN"]
    Gp[:L, M + 1:, N + 1:] = G[:L, rM, rN] * c["MN"]
    Gp[L + 1:, M + 1:, N + 1:] = G[rL, rM, rN] * c["LMN"]
    return Gp


def generate_circulant_tensor(dx: float, ko: float, L: int, M: int, N: int, fl_no_fft: int = 0):
    """lse_generate_circulant_tensor(dx, ko, L, M, N, fl_no_fft) -> (fN_all, st_sparse_precon)."""
    G, st = green_tensor(dx, L, M, N, ko)
    Gp = circulant_embed(G)
    if fl_no_fft:
        return Gp, st
    fN = sfft.fftn(Gp, axes=(0, 1, 2), workers=WORKERS)     # fft_operator.m
    return np.asfortranarray(fN), st
