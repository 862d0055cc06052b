"""Native panel numbering / incidence / port handling vs the oracle, bit-exact (CPU only)."""
import numpy as np
import pytest

from conftest import golden_vhr_text
from oracle import structure as ostruct
from oracle import vhr


@pytest.fixture(scope="module")
def S():
    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import structure

    return structure


def cases():
    from voxhenry_gb300 import geometry

    inp = vhr.read_vhr_text(golden_vhr_text("straight_cond1_len30.0u_wid10.0u_dist20.0u.vhr"))
    yield "numex1", inp.sigma_e, None, inp.dx, inp.pnt_lft, inp.pnt_rght, inp.pnt_well_cond
    inp = vhr.read_vhr_text(golden_vhr_text("wire_len50.0u_dia10.0u.vhr"))
    yield "numex2", inp.sigma_e, None, inp.dx, inp.pnt_lft, inp.pnt_rght, inp.pnt_well_cond
    for shape, seed in (((7, 6, 5), 1), ((12, 9, 4), 2), ((3, 3, 3), 3)):
        w = geometry.random_blob(shape, fill=0.55, seed=seed)
        yield f"blob{shape}", w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght, None
    w = geometry.two_bars(L=24, M=14, N=6, xr=(2, 22), zr=(1, 4), y1=(2, 5), y2=(9, 12))
    yield "two_bars", w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght, None


@pytest.mark.parametrize("case", list(cases()), ids=lambda c: c[0])
def test_setup_matches_oracle(S, case):
    name, sigma, lam, dx, lft, rgt, well = case
    ref = ostruct.build_system(sigma, lam, dx, lft, rgt, well)
    prob = S.build_problem(sigma, lam, dx, lft, rgt, well)
    np.testing.assert_array_equal(prob.idxS, ref.idxS)
    apid, nn = S.panel_ids(prob.idxS, *sigma.shape)
    np.testing.assert_array_equal(apid, ref.all_panels_ids)
    assert nn == ref.num_nodes
    Ae = S.incidence(apid, nn)
    assert (Ae != ref.Ae_full).nnz == 0
    assert prob.Ar.shape == ref.Ar.shape and (prob.Ar != ref.Ar).nnz == 0
    np.testing.assert_array_equal(prob.rhs, ref.rhs)


def test_spiral_and_ring_build(S):
    from voxhenry_gb300 import geometry

    for w in (geometry.square_spiral(), geometry.ring(L=128, M=128, N=8, radius=40, width=6, z0=1)):
        prob = S.problem_from_workload(w)
        assert prob.rhs.shape[1] == 1 and prob.Ar.shape[1] == 5 * prob.idxS.size
        assert np.count_nonzero(prob.rhs) > 0


def test_factor_share_groups_and_a_inv():
    """Factor sharing across frequencies (executer.factor_share_groups): A_inv per class equals the
    oracle's a_inv_diag, and groups break where A_inv moves by more than share_tol."""
    from oracle import circulant, solver
    from oracle import structure as ostruct
    from voxhenry_gb300 import executer, geometry

    w = geometry.two_bars(L=16, M=10, N=5, xr=(1, 15), zr=(1, 3), y1=(1, 3), y2=(6, 8))
    S = ostruct.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    _, st2 = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    P = executer.Problem(S.L, S.M, S.N, S.dx, w.sigma_e, None, S.idxS, S.Ar, S.rhs, None, st2)
    freqs = np.logspace(3, 10, 15)
    A = [executer.a_inv_classes(P, f) for f in freqs]
    for f, a in zip(freqs[::7], A[::7]):
        om = 2 * np.pi * f
        zr, _ = solver.z_arrays(w.sigma_e, None, om)
        ref = solver.a_inv_diag(S.dx, zr, None, S.idxS, 1j * om * solver.MU0 * st2)
        nv = a.shape[0]
        np.testing.assert_allclose(np.concatenate([a[:, 0], a[:, 0], a[:, 0], a[:, 1], a[:, 2]]), ref, rtol=1e-14)
    for tol in (0.0, 1e-8, 1e-4, 1e-2, 10.0):
        rep = executer.factor_share_groups(A, tol)
        assert rep[0] == 0 and np.all(np.diff(rep) >= 0) and np.all(rep <= np.arange(len(freqs)))
        for i, r in enumerate(rep):
            assert np.max(np.abs(A[i] - A[r]) / A[r]) <= tol
    assert len(np.unique(executer.factor_share_groups(A, 0.0))) == len(freqs)
    assert len(np.unique(executer.factor_share_groups(A, 10.0))) == 1
    assert 1 < len(np.unique(executer.factor_share_groups(A, 1e-4))) < len(freqs)


def test_grid_padding_to_fft_lengths_keeps_the_system():
    """A grid with a prime dimension (47) is grown with empty voxels to 7-smooth dimensions when the
    tensor is left to the device; the reduced incidence matrix and the RHS are unchanged."""
    from voxhenry_gb300 import geometry, structure

    assert [structure.smooth7(n) for n in (1, 11, 13, 47, 49, 97, 128)] == [1, 12, 14, 48, 49, 98, 128]
    w = geometry.two_bars(L=47, M=13, N=5, xr=(1, 45), zr=(1, 4), y1=(1, 4), y2=(8, 11))
    P0 = structure.build_problem(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght, tensor=(np.zeros(1), np.zeros(3)))
    P1 = structure.build_problem(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    assert (P1.L, P1.M, P1.N) == (48, 14, 5) and P1.meta["grid_padded_from"] == (47, 13, 5)
    assert (P0.Ar != P1.Ar).nnz == 0 and np.array_equal(P0.rhs, P1.rhs)
    assert np.array_equal(P0.idxS.size, P1.idxS.size)
