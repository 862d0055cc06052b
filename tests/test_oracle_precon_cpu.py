"""Oracle preconditioner variants against each other on CPU: 'schur_gmres' with a tight inner
tolerance applies the exact S^-1 of 'schur_invert' (lse_sparse_precon_multiply.m:26-46 vs :61-117)."""
import numpy as np

from oracle import circulant, solver, structure
from voxhenry_gb300 import geometry


def test_schur_gmres_tight_equals_schur_invert():
    w = geometry.random_blob((8, 6, 5), fill=0.7, seed=3)
    S = structure.build_system(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght)
    _, st2 = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    om = 2 * np.pi * 1e9
    z_real, _ = solver.z_arrays(w.sigma_e, None, om)
    st = 1j * om * solver.MU0 * st2
    inv = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, None, S.idxS, st, S.Ar)
    gm = solver.SparsePrecon("schur_gmres").prepare(S.dx, z_real, None, S.idxS, st, S.Ar)
    gm.prectol = 1e-13
    rng = np.random.default_rng(1)
    x = rng.standard_normal(S.n) + 1j * rng.standard_normal(S.n)
    a, b = gm.multiply(x), inv.multiply(x)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-9
    gm.prectol = 0.1
    c = gm.multiply(x)
    assert 1e-9 < np.linalg.norm(c - b) / np.linalg.norm(b) < 0.5   # a loose inner solve is inexact
