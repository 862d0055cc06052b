"""Current post-processing on the device (voxhenry_gb300.postprocess) vs the oracle's restatement of
post_obtain_curr_coefs_on_grid.m and post_obtain_currs_on_nodes.m."""
import numpy as np
import pytest

from oracle import circulant, postprocess as opost, solver
from oracle import structure as ostruct

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import executer, geometry, postprocess

    w = geometry.two_bars(L=20, M=12, N=6, xr=(1, 19), zr=(1, 4), y1=(1, 4), y2=(7, 10))
    S = ostruct.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    fN, st = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    P = executer.Problem(S.L, S.M, S.N, S.dx, w.sigma_e, None, S.idxS, S.Ar, S.rhs, fN, st)
    out = executer.Sweep(P, np.array([2.5e9])).prepare().solve(restart=50, tol=1e-10, maxit=10)
    L, M, N = S.L, S.M, S.N
    ii, jj, kk = np.meshgrid(np.arange(L), np.arange(M), np.arange(N), indexing="ij")
    r = np.stack([(ii + 0.5) * S.dx, (jj + 0.5) * S.dx, (kk + 0.5) * S.dx], axis=-1)
    return w, S, out["x"], r, postprocess


def test_curr_coefs_on_grid(setup):
    w, S, X, r, post = setup
    rng = np.random.default_rng(3)
    Xb = np.concatenate([X, rng.standard_normal(X.shape) + 1j * rng.standard_normal(X.shape)])
    got = post.post_obtain_curr_coefs_on_grid(Xb, w.sigma_e)
    for b in range(Xb.shape[0]):
        ref = opost.post_obtain_curr_coefs_on_grid(Xb[b], w.sigma_e)
        for c in range(5):
            np.testing.assert_array_equal(got[c][b], ref[c])
        assert got[5][b] == ref[5] and got[6][b] == ref[6]


def test_currs_on_nodes(setup):
    w, S, X, r, post = setup
    rng = np.random.default_rng(4)
    Xb = np.concatenate([X, rng.standard_normal(X.shape) + 1j * rng.standard_normal(X.shape)])
    got = post.post_obtain_currs_on_nodes(Xb, S.Ae_only_leaving, S.Ae_only_entering_bndry, r, w.sigma_e, S.dx)
    for b in range(Xb.shape[0]):
        ref = opost.post_obtain_currs_on_nodes(Xb[b], S.Ae_only_leaving, S.Ae_only_entering_bndry, r, w.sigma_e, S.dx)
        for a in range(3):
            assert got[b][a].shape == ref[a].shape and got[b][a].shape[0] > 0
            np.testing.assert_array_equal(got[b][a][:, :3], ref[a][:, :3])
            np.testing.assert_allclose(got[b][a][:, 3], ref[a][:, 3], rtol=1e-13, atol=1e-13 * np.abs(ref[a][:, 3]).max())

