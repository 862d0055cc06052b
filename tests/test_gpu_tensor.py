"""Circulant Green tensor generated on the GPU vs the oracle's lse_generate_circulant_tensor."""
import numpy as np
import pytest

from oracle import circulant

pytestmark = pytest.mark.gpu

TENSOR_TOL = 1e-12     # max |difference| / max |fN_all|, per component


@pytest.fixture(scope="module")
def S():
    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import structure

    return structure


@pytest.mark.parametrize("shape,dx", [((2, 2, 2), 1e-6), ((6, 5, 4), 0.5e-6), ((12, 3, 7), 1e-6), ((20, 10, 10), 2e-6),
                                      ((5, 5, 5), 1e-6), ((9, 3, 2), 1e-8)])
def test_tensor_matches_oracle(S, shape, dx):
    L, M, N = shape
    fN, st = S.circulant_tensor(L, M, N, dx)
    ref, st_ref = circulant.generate_circulant_tensor(dx, 1.0, L, M, N)
    for k in range(7):
        scale = np.abs(ref[..., k]).max()
        assert np.abs(fN[..., k] - ref[..., k]).max() <= TENSOR_TOL * scale, k
    np.testing.assert_allclose(st, st_ref, rtol=1e-13)


def test_generated_geometry_solve(S):
    """Sweep on a device-generated tensor == Sweep on the oracle's tensor (R, L to 1e-10)."""
    from voxhenry_gb300 import executer, geometry

    w = geometry.bar(L=16, M=6, N=4, dx=1e-6)
    p_dev = S.problem_from_workload(w)
    fN, st = circulant.generate_circulant_tensor(w.dx, 1.0, 16, 6, 4)
    p_host = S.problem_from_workload(w, tensor=(fN, st))
    freqs = np.array([1e4, 3e9])
    a = executer.Sweep(p_dev, freqs).prepare().solve(tol=1e-12)
    b = executer.Sweep(p_host, freqs).prepare().solve(tol=1e-12)
    np.testing.assert_allclose(a["R"], b["R"], rtol=1e-10)
    np.testing.assert_allclose(a["L"], b["L"], rtol=1e-10)
