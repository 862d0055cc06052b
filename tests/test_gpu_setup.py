"""Panel numbering and Ae built on the device (vh_setup_device) vs the oracle, bit-exact.

Covers lse_generate_panelIDs.m:25-172 and lse_compute_Ae_matrix.m:205-264: the device builds the ids
by prefix sums over each axis's scan order; the sequential numbering of the reference must come out
exactly, on blobs, edge cases (an empty grid, one voxel, a full grid, runs that touch the grid's
faces) and a grid of more than 2048^2 cells, where the scan of block sums recurses."""
import numpy as np
import pytest

from oracle import structure as ostruct

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import structure, vie

    ctx = vie.Context(0)
    yield structure, ctx
    ctx.close()


def _idx(occ):
    return (np.flatnonzero(occ.ravel(order="F")) + 1).astype(np.int64)


def grids():
    rng = np.random.default_rng(7)
    yield "empty", np.zeros((4, 3, 2), bool)
    one = np.zeros((5, 4, 3), bool)
    one[2, 1, 1] = True
    yield "one_voxel", one
    yield "full", np.ones((9, 7, 5), bool)
    corner = np.zeros((6, 5, 4), bool)
    corner[-1, :, :] = True
    corner[:, -1, 0] = True
    corner[0, 0, :] = True
    yield "faces", corner
    yield "line_x", np.ones((33, 1, 1), bool)
    for shape, fill in (((7, 6, 5), 0.55), ((31, 17, 9), 0.3), ((64, 48, 12), 0.8)):
        yield f"blob{shape}", rng.random(shape) < fill
    big = rng.random((256, 256, 80)) < 0.6        # 5.2 M cells: three scan blocks levels deep
    yield "big_256x256x80", big


@pytest.mark.parametrize("case", list(grids()), ids=lambda c: c[0])
def test_device_setup_matches_oracle(env, case):
    S, ctx = env
    name, occ = case
    L, M, N = occ.shape
    idxS = _idx(occ)
    apid, nn, Ae = S.setup_device(ctx, idxS, L, M, N)
    if idxS.size == 0:
        assert nn == 0 and apid.shape == (0, 6)
        return
    ref_ap, ref_nn = ostruct.generate_panel_ids(idxS, L, M, N)
    np.testing.assert_array_equal(apid, ref_ap)
    assert nn == ref_nn
    host_ap, host_nn = S.panel_ids(idxS, L, M, N)
    np.testing.assert_array_equal(apid, host_ap)
    ref_Ae = ostruct.compute_Ae(ref_ap, ref_nn)[0]
    assert Ae.shape == ref_Ae.shape
    np.testing.assert_array_equal(Ae.indptr, ref_Ae.indptr)
    np.testing.assert_array_equal(Ae.indices, ref_Ae.indices)
    np.testing.assert_array_equal(Ae.data, ref_Ae.data)


def test_device_setup_without_incidence_and_errors(env):
    S, ctx = env
    occ = np.random.default_rng(3).random((10, 8, 6)) < 0.5
    idxS = _idx(occ)
    apid, nn, Ae = S.setup_device(ctx, idxS, 10, 8, 6, with_incidence=False)
    assert Ae is None
    ref_ap, ref_nn = ostruct.generate_panel_ids(idxS, 10, 8, 6)
    np.testing.assert_array_equal(apid, ref_ap)
    assert nn == ref_nn
    from voxhenry_gb300 import _lib

    for bad in (idxS[::-1].copy(), np.array([0, 1], np.int64), np.array([1, 10 * 8 * 6 + 1], np.int64)):
        with pytest.raises(_lib.VHError):
            S.setup_device(ctx, bad, 10, 8, 6)
    # the context stays usable after a rejected call
    apid2, nn2, _ = S.setup_device(ctx, idxS, 10, 8, 6)
    np.testing.assert_array_equal(apid2, ref_ap)


def test_problem_built_on_device_equals_host(env):
    S, ctx = env
    from voxhenry_gb300 import geometry

    w = geometry.random_blob((12, 9, 6), fill=0.6, seed=5)
    host = S.problem_from_workload(w)
    dev = S.problem_from_workload(w, ctx=ctx)
    np.testing.assert_array_equal(dev.idxS, host.idxS)
    assert dev.Ar.shape == host.Ar.shape and (dev.Ar != host.Ar).nnz == 0
    np.testing.assert_array_equal(dev.rhs, host.rhs)
