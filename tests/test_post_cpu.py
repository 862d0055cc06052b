"""Host side of the post-processing: the incidence split against the oracle's compute_Ae
(lse_compute_Ae_matrix.m:94-113), and the oracle's node-current restatement against a direct reading
of post_obtain_currs_on_nodes.m on a one-voxel case."""
import numpy as np
import scipy.sparse as sp

from oracle import postprocess as opost
from oracle import structure as ostruct
from voxhenry_gb300 import geometry, postprocess


def test_incidence_split_matches_oracle():
    w = geometry.two_bars(L=20, M=12, N=6, xr=(1, 19), zr=(1, 4), y1=(1, 4), y2=(7, 10))
    S = ostruct.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    Ae, lv, en = postprocess.incidence_split(S.all_panels_ids, S.num_nodes)
    assert (Ae != S.Ae_full).nnz == 0
    assert (lv != S.Ae_only_leaving).nnz == 0 and lv.nnz > 0
    assert (en != S.Ae_only_entering_bndry).nnz == 0 and en.nnz > 0


def test_oracle_nodes_one_voxel():
    # one voxel: node ids of its six panels are 1..6 (-x +x -y +y -z +z) and a 7th for the centre
    Mc = np.ones((1, 1, 1))
    apid = np.array([[1, 2, 3, 4, 5, 6]], dtype=np.int64)
    Ae, lv, en = ostruct.compute_Ae(apid, 7)
    x = np.array([1.0 + 2j, 3.0 - 1j, -2.0 + 0.5j, 0.25, -0.75j])
    r = np.full((1, 1, 1, 3), 0.5)
    dx = 1.0
    nx, ny, nz = opost.post_obtain_currs_on_nodes(x, lv, en, r, Mc, dx)
    xn = -(lv @ x) + en @ x
    # each aligned list: the leaving (minus-side) node first, then the entering (plus-side) node
    for out, c in ((nx, 0), (ny, 1), (nz, 2)):
        assert out.shape == (2, 4)
        minus, plus = out[0], out[1]
        assert minus[c].real == 0.0 and plus[c].real == 1.0
        np.testing.assert_allclose([minus[3], plus[3]], [xn[2 * c], xn[2 * c + 1]])
    grids = opost.post_obtain_curr_coefs_on_grid(x, Mc)
    assert [g[0, 0, 0] for g in grids[:5]] == list(x)
    assert grids[5] == np.abs(x[:3]).min() and grids[6] == np.abs(x[:3]).max()
