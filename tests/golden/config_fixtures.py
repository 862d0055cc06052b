"""Oracle fixtures of the four benchmark configurations (test infrastructure).

Each fixture holds what the oracle (the NumPy/SciPy restatement of the reference's FP64 path,
oracle/solver.py) computes on one of the seeded synthetic workloads of voxhenry_gb300.geometry:
  * Y, Z, R and L per frequency (VoxHenry_executer.m:311-328), with GMRES run to tol 1e-14 so that
    they are the converged values;
  * the sensitivity of each point: the relative change of R, L and x between that solve and a second
    one at tol 1e-12.  Both stop where the true residual has reached its FP64 floor, so the change is
    what the conditioning of the point leaves undetermined (at the spiral's 20 GHz point R moves by
    1.1e-8: R there is a small real part of a mostly inductive impedance);
  * fingerprints of every solution x (current coefficients and node potentials separately), small
    enough to commit: a strided sample, the 2-norms of fixed blocks and a Gaussian sketch G x with a
    seeded K x n matrix G.  For two solutions, |G (x1 - x2)| / |G x2| estimates |x1 - x2| / |x2|
    within a factor of about 1 +- 2/sqrt(K) (Johnson-Lindenstrauss), so a GPU solution can be compared
    with the oracle's norm-wise without storing x itself (up to 12 MB per right-hand side at the ring);
  * for the straight bar, also the solve at its own GMRES settings (tol 1e-8, restart 50, maxit 10):
    x fingerprints, iteration counts and R, L.

tests/golden/make_config_fixtures.py writes them (config_<name>.npz); the parity tests read them.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# frequencies (indices into the workload's own list) that the oracle solves for each configuration:
# all 8 of the bar; 4 of the spiral's 32 from 1 MHz to the top frequency 20 GHz; 4 of the two bars'
# 16 (x 2 ports); the first and last of the ring's 16
CONFIGS = {
    "bar_64x16x16": {"freq_idx": list(range(8)), "config_tol": 1e-8},
    "square_spiral_256x256x8": {"freq_idx": [0, 10, 21, 31]},
    "two_bars_128x64x32": {"freq_idx": [0, 5, 10, 15]},
    "ring_512x512x16": {"freq_idx": [0, 15]},
}
TOL_REF = 1e-14        # GMRES tolerance of the converged oracle values
TOL_SENS = 1e-12       # the second solve that measures each point's sensitivity
RESTART = 50
MAXIT_REF = 40
SKETCH_SEED = 20261203
SKETCH_K = 64
SAMPLE_POINTS = 512    # strided samples per block (currents, potentials)
NBLOCKS = 64           # block 2-norms per block


def path(name: str) -> str:
    return os.path.join(HERE, f"config_{name}.npz")


def sketch_matrix_apply(X: np.ndarray, seed: int = SKETCH_SEED, k: int = SKETCH_K, chunk: int = 65536) -> np.ndarray:
    """G @ X.T for rows X (B, n): G is K x n standard normal, drawn in column chunks of `chunk` from
    numpy.random.default_rng(seed) (the same draw for every caller)."""
    X = np.atleast_2d(X)
    n = X.shape[1]
    rng = np.random.default_rng(seed)
    out = np.zeros((X.shape[0], k), dtype=np.complex128)
    for c0 in range(0, n, chunk):
        c1 = min(n, c0 + chunk)
        G = rng.standard_normal((k, c1 - c0))
        out += X[:, c0:c1] @ G.T
    return out


def sample_idx(n: int) -> np.ndarray:
    return np.unique(np.linspace(0, n - 1, min(n, SAMPLE_POINTS)).astype(np.int64))


def block_norms(X: np.ndarray) -> np.ndarray:
    X = np.atleast_2d(X)
    edges = np.linspace(0, X.shape[1], NBLOCKS + 1).astype(np.int64)
    return np.stack([np.linalg.norm(X[:, a:b], axis=1) for a, b in zip(edges[:-1], edges[1:])], axis=1)


def fingerprint(X: np.ndarray, nc: int) -> dict:
    """Fingerprints of solutions X (B, n): per part (currents x[:nc], potentials x[nc:]) a strided
    sample, block norms, the full 2-norm and the sketch."""
    X = np.atleast_2d(X)
    out = {}
    for part, (a, b) in {"curr": (0, nc), "phi": (nc, X.shape[1])}.items():
        Xp = X[:, a:b]
        idx = sample_idx(Xp.shape[1])
        out[f"{part}_idx"] = idx
        out[f"{part}_sample"] = Xp[:, idx]
        out[f"{part}_blocks"] = block_norms(Xp)
        out[f"{part}_norm"] = np.linalg.norm(Xp, axis=1)
        out[f"{part}_sketch"] = sketch_matrix_apply(Xp, seed=SKETCH_SEED + (0 if part == "curr" else 1))
    return out


def compare(X: np.ndarray, nc: int, fx: dict, prefix: str = "x_") -> dict:
    """Relative differences of solutions X (B, n) against stored fingerprints (keys prefix + ...):
    per part, the sketch estimate of |x - x_ref| / |x_ref| (max over rows), the exact relative norm
    difference, the sampled max |x - x_ref| / max|x_ref| and the block-norm relative difference."""
    X = np.atleast_2d(X)
    res = {}
    for part, (a, b) in {"curr": (0, nc), "phi": (nc, X.shape[1])}.items():
        Xp = X[:, a:b]
        sk = sketch_matrix_apply(Xp, seed=SKETCH_SEED + (0 if part == "curr" else 1))
        skr = fx[prefix + f"{part}_sketch"]
        res[f"{part}_sketch"] = float(np.max(np.linalg.norm(sk - skr, axis=1) / np.linalg.norm(skr, axis=1)))
        nr = fx[prefix + f"{part}_norm"]
        res[f"{part}_norm"] = float(np.max(np.abs(np.linalg.norm(Xp, axis=1) - nr) / nr))
        idx = fx[prefix + f"{part}_idx"]
        smp = fx[prefix + f"{part}_sample"]
        res[f"{part}_sample"] = float(np.max(np.abs(Xp[:, idx] - smp).max(axis=1) / np.abs(smp).max(axis=1)))
        bl = fx[prefix + f"{part}_blocks"]
        bg = block_norms(Xp)
        res[f"{part}_blocks"] = float(np.max(np.abs(bg - bl) / np.maximum(bl, 1e-300 + bl.max(axis=1, keepdims=True) * 1e-3)))
    return res


def load(name: str) -> dict:
    with np.load(path(name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def bound(fx: dict, key: str, base: float, factor: float = 10.0) -> np.ndarray:
    """Per-frequency comparison bound for R or L: base, or `factor` times the point's own sensitivity
    (sens_R / sens_L) where the conditioning leaves more undetermined."""
    return np.maximum(base, factor * fx["sens_" + key])
