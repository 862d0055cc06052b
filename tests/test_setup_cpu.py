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
