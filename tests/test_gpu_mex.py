"""The MATLAB / Octave gateway on the GPU, driven as VoxHenry_executer.m drives the reference
(lse_matvect_mult, lse_sparse_precon_prepare / _multiply, pgmres), in both complex layouts, against
the oracle: the FP64 product within 1e-12, the preconditioner within 1e-10, the solution within 1e-9."""
import os
import shutil
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "mex_stub"))
import gateway  # noqa: E402

from oracle import circulant, solver, structure  # noqa: E402

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc builds the gateway")]


@pytest.fixture(scope="module", params=[False, True], ids=["split", "interleaved"])
def gw(request, tmp_path_factory):
    import __graft_entry__

    __graft_entry__.build()
    g = gateway.Gateway(gateway.build(str(tmp_path_factory.mktemp("mex")), request.param))
    yield g
    g("reset", nargout=0)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_executer_sequence_matches_oracle(gw):
    from voxhenry_gb300 import geometry

    # a connected random conductor (an island of voxels would leave S singular on it)
    w = geometry.random_blob((10, 7, 6), fill=0.7, seed=5)
    S = structure.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    fN2, st2 = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    for f in (2.5e9, 2e10):
        om = 2 * np.pi * f
        jwmu = 1j * om * solver.MU0
        fN = jwmu * fN2
        st = jwmu * st2
        z_real, _ = solver.z_arrays(w.sigma_e, None, om)
        idxS5 = S.idxS5.astype(np.float64)
        rng = np.random.default_rng(int(f) % 97)
        J = rng.standard_normal(S.n) + 1j * rng.standard_normal(S.n)
        # lse_matvect_mult
        y = gw("matvec", J, fN, S.Ar, z_real, np.zeros((0, 0)), S.dx, idxS5)
        yo = solver.lse_matvect_mult(J, fN, S.Ar, z_real, None, S.dx, S.idxS5)
        assert rel(y, yo) < 1e-12
        # lse_sparse_precon_prepare / lse_sparse_precon_multiply
        gw("precon_prepare", S.dx, z_real, np.zeros((0, 0)), S.idxS.astype(np.float64), st, S.Ar, "schur_invert",
           nargout=0)
        ref = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, None, S.idxS, st, S.Ar)
        assert rel(gw("precon_multiply", J, 0.1), ref.multiply(J)) < 1e-10
        # pgmres(@(J)fACPU(J), rhs, inner_it, tol, outer_it, @(x)fPCPU(x)): the whole loop on the device
        b = S.rhs[:, 0].astype(complex)
        x, flag, relres, it, resvec = gw("gmres", b, 100, 1e-12, 10, 0.0, np.zeros((0, 0)), fN, S.Ar, z_real,
                                         np.zeros((0, 0)), S.dx, idxS5, 1.0, nargout=5)
        Aref = lambda v: solver.lse_matvect_mult(v, fN, S.Ar, z_real, None, S.dx, S.idxS5)
        xo, flag_o, relres_o, it_o, resvec_o = solver.pgmres(Aref, b, 100, 1e-12, 10, ref.multiply)
        assert rel(x, xo) < 1e-9
        assert int(np.ravel(flag)[0]) == flag_o and float(np.ravel(relres)[0]) < 1e-10
        assert np.ravel(it).tolist() == [it_o[0], it_o[1]]
        np.testing.assert_allclose(np.ravel(resvec)[:3], resvec_o[:3], rtol=1e-6)
