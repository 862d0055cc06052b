"""Preconditioner, (F)GMRES and R/L extraction on the GPU vs the CPU oracle and the reference's results."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_vhr_text
from oracle import circulant, solver, structure, vhr

pytestmark = pytest.mark.gpu

PRECON_TOL = 1e-10     # preconditioner apply, relative 2-norm (different exact factorisation of S)


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import executer, vie

    return vie, executer


def problem_of(w):
    from voxhenry_gb300.executer import Problem

    S = structure.build_system(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght)
    fN, st = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    P = Problem(S.L, S.M, S.N, S.dx, w.sigma_e, w.lambdaL, S.idxS, S.Ar, S.rhs, fN, st)
    return S, P


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def assert_port_matrix_close(a, b, rtol):
    """Per frequency, |a - b| <= rtol * max|b| over the port matrix (off-diagonal mutual terms of
    decoupled conductors sit at the rounding floor of the diagonal ones)."""
    for f in range(b.shape[0]):
        scale = np.abs(b[f]).max()
        assert np.abs(a[f] - b[f]).max() <= rtol * scale, (f, a[f], b[f])


@pytest.fixture(scope="module")
def blob(lib):
    from voxhenry_gb300 import geometry

    w = geometry.random_blob((10, 7, 6), fill=0.7, seed=5)
    return w, *problem_of(w)


@pytest.mark.parametrize("f", [1e3, 1e8, 2e10])
def test_precon_apply_matches_oracle(lib, blob, f):
    vie, ex = lib
    w, S, P = blob
    om = 2 * np.pi * f
    jwmu = 1j * om * solver.MU0
    z_real, z_imag = solver.z_arrays(w.sigma_e, None, om)
    ref = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, z_imag, S.idxS, jwmu * P.st2, S.Ar)
    g = vie.Geometry(P.fN_all2, S.Ar, z_real, None, S.dx, S.idxS)
    pc = g.precon(jwmu * P.st2)
    rng = np.random.default_rng(7)
    X = rng.standard_normal((3, S.n)) + 1j * rng.standard_normal((3, S.n))
    Y = vie.apply_precons(g, [pc], X)
    for k in range(3):
        assert rel(Y[k], ref.multiply(X[k])) < PRECON_TOL
    st = pc.stats()
    assert st["fronts"] >= 1 and st["nnz_factor"] > 0


def test_precon_apply_spiral_matches_oracle(lib):
    """A 2-turn spiral: many fronts with partial 32-column blocks and empty separators."""
    vie, ex = lib
    from voxhenry_gb300 import geometry

    w = geometry.square_spiral(L=96, M=96, N=4, turns=2, thick=2)
    S, P = problem_of(w)
    f = 3e9
    om = 2 * np.pi * f
    jwmu = 1j * om * solver.MU0
    z_real, _ = solver.z_arrays(w.sigma_e, None, om)
    ref = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, None, S.idxS, jwmu * P.st2, S.Ar)
    g = vie.Geometry(P.fN_all2, S.Ar, z_real, None, S.dx, S.idxS)
    pcs = g.precons(np.stack([jwmu * P.st2] * 3))
    rng = np.random.default_rng(17)
    X = rng.standard_normal((3, S.n)) + 1j * rng.standard_normal((3, S.n))
    Y = vie.apply_precons(g, pcs, X)
    for k in range(3):
        assert np.all(np.isfinite(Y[k]))
        assert rel(Y[k], ref.multiply(X[k])) < PRECON_TOL


def test_dropin_calls_match_oracle(lib, blob):
    """lse_sparse_precon_prepare / lse_sparse_precon_multiply / pgmres with the reference's arguments."""
    vie, ex = lib
    w, S, P = blob
    f = 2.5e9
    om = 2 * np.pi * f
    jwmu = 1j * om * solver.MU0
    fN = jwmu * P.fN_all2
    st = jwmu * P.st2
    z_real, z_imag = solver.z_arrays(w.sigma_e, None, om)
    ref = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, z_imag, S.idxS, st, S.Ar)
    vie.lse_sparse_precon_prepare(S.dx, z_real, z_imag, S.idxS, st, S.nodeid_4_grnd, S.nodeid_4_injectcurr, S.Ar)
    x = np.random.default_rng(3).standard_normal(S.n) + 0j
    assert rel(vie.lse_sparse_precon_multiply(x, S.Ar, None, None, 0.1), ref.multiply(x)) < PRECON_TOL
    A = vie.matvec_handle(fN, S.Ar, z_real, z_imag, S.dx, S.idxS5)
    b = S.rhs[:, 0].astype(complex)
    xg, flag, relres, it, resvec = vie.pgmres(A, b, 100, 1e-12, 10, vie.precon_handle())
    Aref = lambda J: solver.lse_matvect_mult(J, fN, S.Ar, z_real, z_imag, S.dx, S.idxS5)
    xo, flag_o, relres_o, it_o, resvec_o = solver.pgmres(Aref, b, 100, 1e-12, 10, ref.multiply)
    assert rel(xg, xo) < 1e-9
    assert abs(len(resvec) - len(resvec_o)) <= 1
    np.testing.assert_allclose(resvec[:3], resvec_o[:3], rtol=1e-6)
    assert relres < 1e-10 and flag == flag_o


def test_fpgmres_matches_oracle(lib, blob):
    vie, ex = lib
    w, S, P = blob
    f = 1e9
    om = 2 * np.pi * f
    jwmu = 1j * om * solver.MU0
    z_real, _ = solver.z_arrays(w.sigma_e, None, om)
    g = vie.Geometry(P.fN_all2, S.Ar, z_real, None, S.dx, S.idxS)
    pc = g.precon(jwmu * P.st2)
    b = S.rhs[:, 0].astype(complex)
    out = g.solve(b[None], pcs=[pc], scale=jwmu, restart=30, tol=1e-11, maxit=10, flexible=True)
    ref = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, None, S.idxS, jwmu * P.st2, S.Ar)
    Aref = lambda J: solver.lse_matvect_mult(J, jwmu * P.fN_all2, S.Ar, z_real, None, S.dx, S.idxS5)
    xo, *_ = solver.fpgmres(Aref, b, 30, 1e-11, 10, ref.multiply)
    assert rel(out["x"][0], xo) < 1e-9


def test_sweep_rl_matches_oracle_and_batching_invariant(lib):
    """All frequencies x ports in one batch == the oracle per frequency; one RHS alone == in the batch."""
    vie, ex = lib
    from voxhenry_gb300 import geometry

    w = geometry.two_bars(L=24, M=14, N=6, xr=(2, 22), zr=(1, 4), y1=(2, 5), y2=(9, 12))
    S, P = problem_of(w)
    freqs = np.array([1e3, 1e7, 5e9])
    sw = ex.Sweep(P, freqs).prepare()
    out = sw.solve(restart=50, tol=1e-12, maxit=10)
    ref = solver.solve_frequencies(S, P.fN_all2, P.st2, freqs, restart=50, tol=1e-12)
    assert_port_matrix_close(out["R"], ref["R"], 1e-9)
    assert_port_matrix_close(out["L"], ref["L"], 1e-9)
    # batching invariance: the last frequency's port-1 solve alone, bitwise
    g = sw.geom
    k = 2 * P.num_ports
    alone = g.solve(P.rhs[:, 0].astype(complex)[None], pcs=[sw.pcs[2]], scale=1j * 2 * np.pi * freqs[2] * solver.MU0,
                    restart=50, tol=1e-12, maxit=10)
    assert np.array_equal(alone["x"][0], out["x"][k])


def test_mixed_precision_rl(lib):
    """complex64 FFT inside FP64 refinement: R, L within 1e-6 of the FP64 oracle."""
    vie, ex = lib
    from voxhenry_gb300 import geometry

    w = geometry.bar(L=24, M=6, N=6, dx=0.5e-6)
    S, P = problem_of(w)
    freqs = np.array([1e3, 1e8, 1e10])
    sw = ex.Sweep(P, freqs).prepare()
    out = sw.solve(restart=50, tol=1e-10, maxit=10, prec="fp32")
    ref = solver.solve_frequencies(S, P.fN_all2, P.st2, freqs, restart=50, tol=1e-12)
    assert_port_matrix_close(out["R"], ref["R"], 1e-6)
    assert_port_matrix_close(out["L"], ref["L"], 1e-6)
    out64 = sw.solve(restart=50, tol=1e-12, maxit=10)
    assert_port_matrix_close(out64["R"], ref["R"], 1e-9)
    assert_port_matrix_close(out64["L"], ref["L"], 1e-9)


def test_numex1_matches_reference_results(lib):
    """The reference's numex1 input: GPU R, L vs results_numex1_straight_conductor/data_R_jL_mat.mat."""
    vie, ex = lib
    gold = np.load(os.path.join(GOLDEN, "reference_results.npz"))
    inp = vhr.read_vhr_text(golden_vhr_text("straight_cond1_len30.0u_wid10.0u_dist20.0u.vhr"))
    from voxhenry_gb300 import geometry

    w = geometry.Workload("numex1", inp.sigma_e, inp.dx, inp.pnt_lft, inp.pnt_rght, inp.freq)
    S, P = problem_of(w)
    sel = [0, 24, 37, 40]        # 1 Hz, 1 MHz, 2.5 GHz, 10 GHz
    freqs = gold["numex1_freq"][sel]
    out = ex.Sweep(P, freqs).prepare().solve(restart=100, tol=None, maxit=10)
    RjL = gold["numex1_RjL"][sel]
    np.testing.assert_allclose(out["R"][:, 0, 0], RjL.real, rtol=1e-7)
    np.testing.assert_allclose(out["L"][:, 1 - 1, 0][1:], RjL.imag[1:], rtol=1e-7)
    np.testing.assert_allclose(out["L"][0, 0, 0], RjL.imag[0], rtol=1e-5)   # 1 Hz: L from a 1e-8 part of Z
    x = out["x"][2]
    idx = gold["numex1_x_sample_idx"]
    np.testing.assert_allclose(x[idx], gold["numex1_x_sample"], rtol=0, atol=1e-6 * np.abs(gold["numex1_x_sample"]).max())


def test_precon_double_float_factor(lib, blob):
    """VH_PRECON_SCHUR_INVERT_DF: factor and triangular solves in FP32 pairs (~48 bits): within
    about cond(S) x 4e-15 of the FP64 preconditioner; 1e-10 on this geometry."""
    vie, ex = lib
    w, S, P = blob
    om = 2 * np.pi * 1e9
    jwmu = 1j * om * solver.MU0
    z_real, _ = solver.z_arrays(w.sigma_e, None, om)
    ref = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, None, S.idxS, jwmu * P.st2, S.Ar)
    g = vie.Geometry(P.fN_all2, S.Ar, z_real, None, S.dx, S.idxS)
    pcs = g.precons(np.stack([jwmu * P.st2] * 3), kind="schur_invert_df")
    rng = np.random.default_rng(11)
    X = rng.standard_normal((3, S.n)) + 1j * rng.standard_normal((3, S.n))
    Y = vie.apply_precons(g, pcs, X)
    for k in range(3):
        assert np.all(np.isfinite(Y[k]))
        assert rel(Y[k], ref.multiply(X[k])) < 1e-10


def test_precon_double_float_spiral(lib):
    """The double-float factor on a 2-turn spiral (partial blocks, empty separators, larger condition)."""
    vie, ex = lib
    from voxhenry_gb300 import geometry

    w = geometry.square_spiral(L=96, M=96, N=4, turns=2, thick=2)
    S, P = problem_of(w)
    om = 2 * np.pi * 3e9
    jwmu = 1j * om * solver.MU0
    z_real, _ = solver.z_arrays(w.sigma_e, None, om)
    ref = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, None, S.idxS, jwmu * P.st2, S.Ar)
    g = vie.Geometry(P.fN_all2, S.Ar, z_real, None, S.dx, S.idxS)
    pcs = g.precons(np.stack([jwmu * P.st2] * 2), kind="schur_invert_df")
    rng = np.random.default_rng(17)
    X = rng.standard_normal((2, S.n)) + 1j * rng.standard_normal((2, S.n))
    Y = vie.apply_precons(g, pcs, X)
    for k in range(2):
        assert np.all(np.isfinite(Y[k]))
        assert rel(Y[k], ref.multiply(X[k])) < 1e-8


def test_mixed_precision_double_float_factor_rl(lib):
    """Mixed precision with the double-float Schur factor: R, L within 1e-6 of the oracle, every flag 0."""
    vie, ex = lib
    from voxhenry_gb300 import geometry

    w = geometry.two_bars(L=24, M=14, N=6, xr=(2, 22), zr=(1, 4), y1=(2, 5), y2=(9, 12))
    S, P = problem_of(w)
    freqs = np.array([1e3, 1e8, 1e10])
    sw = ex.Sweep(P, freqs, precon="schur_invert_df").prepare()
    out = sw.solve(restart=50, tol=1e-10, maxit=10, prec="fp32")
    ref = solver.solve_frequencies(S, P.fN_all2, P.st2, freqs, restart=50, tol=1e-12)
    assert np.all(out["flag"] == 0)
    assert_port_matrix_close(out["R"], ref["R"], 1e-6)
    assert_port_matrix_close(out["L"], ref["L"], 1e-6)


def test_mixed_precision_relres_is_the_fp64_residual(lib):
    """Mixed precision updates the residual after the first refinement step with the complex64 product
    of the correction; the reported relres must still be the FP64 residual |b - A x| / |b| to ~1e-11."""
    vie, ex = lib
    from voxhenry_gb300 import geometry

    w = geometry.two_bars(L=24, M=14, N=6, xr=(2, 22), zr=(1, 4), y1=(2, 5), y2=(9, 12))
    S, P = problem_of(w)
    freqs = np.array([1e3, 1e8, 1e10])
    sw = ex.Sweep(P, freqs, precon="schur_invert_df").prepare()
    out = sw.solve(restart=50, tol=1e-10, maxit=10, prec="fp32")
    g = sw.geom
    for k in range(len(out["x"])):
        f = freqs[k // P.num_ports]
        s = 1j * 2 * np.pi * f * solver.MU0
        b = P.rhs[:, k % P.num_ports].astype(complex)
        r = b - g.matvec(out["x"][k], scale=s)
        true_rel = np.linalg.norm(r) / np.linalg.norm(b)
        assert abs(true_rel - out["relres"][k]) < 1e-11
        assert true_rel < 1e-10 + 2e-11 and out["flag"][k] == 0


def test_precon_schur_approx_matches_oracle(lib, blob):
    """'schur_approx' (lse_sparse_precon_prepare.m:71-81, lse_sparse_precon_multiply.m:48-58)."""
    vie, ex = lib
    w, S, P = blob
    om = 2 * np.pi * 3e8
    jwmu = 1j * om * solver.MU0
    z_real, _ = solver.z_arrays(w.sigma_e, None, om)
    ref = solver.SparsePrecon("schur_approx").prepare(S.dx, z_real, None, S.idxS, jwmu * P.st2, S.Ar)
    g = vie.Geometry(P.fN_all2, S.Ar, z_real, None, S.dx, S.idxS)
    pcs = g.precons(np.stack([jwmu * P.st2] * 3), kind="schur_approx")
    rng = np.random.default_rng(23)
    X = rng.standard_normal((3, S.n)) + 1j * rng.standard_normal((3, S.n))
    Y = vie.apply_precons(g, pcs, X)
    for k in range(3):
        assert rel(Y[k], ref.multiply(X[k])) < 1e-12


def test_pgmres_schur_approx_matches_oracle(lib, blob):
    """pgmres with the 'schur_approx' preconditioner through the drop-in calls: the same iterations as
    the oracle (this weak preconditioner does not reach tol here in either; both report flag 1)."""
    vie, ex = lib
    w, S, P = blob
    om = 2 * np.pi * 1e9
    jwmu = 1j * om * solver.MU0
    fN = jwmu * P.fN_all2
    st = jwmu * P.st2
    z_real, _ = solver.z_arrays(w.sigma_e, None, om)
    vie.lse_sparse_precon_prepare(S.dx, z_real, None, S.idxS, st, None, None, S.Ar, kind="schur_approx")
    A = vie.matvec_handle(fN, S.Ar, z_real, None, S.dx, S.idxS5)
    b = S.rhs[:, 0].astype(complex)
    xg, flag, relres, it, resvec = vie.pgmres(A, b, 20, 1e-10, 2, vie.precon_handle())
    ref = solver.SparsePrecon("schur_approx").prepare(S.dx, z_real, None, S.idxS, st, S.Ar)
    Aref = lambda J: solver.lse_matvect_mult(J, fN, S.Ar, z_real, None, S.dx, S.idxS5)
    xo, flag_o, relres_o, it_o, resvec_o = solver.pgmres(Aref, b, 20, 1e-10, 2, ref.multiply)
    assert flag == flag_o
    assert tuple(it) == tuple(it_o) and len(resvec) == len(resvec_o)
    np.testing.assert_allclose(resvec, resvec_o, rtol=1e-6)
    assert abs(relres - relres_o) <= 1e-6 * relres_o
    assert rel(xg, xo) < 1e-8


def test_sharded_sweep_with_gpu_solver(lib):
    """sharding.sweep_distributed with the GPU Sweep solver (one gloo rank on this process) gives the
    same R, L as a direct Sweep over all frequencies."""
    import socket

    import torch.distributed as dist

    vie, ex = lib
    from voxhenry_gb300 import geometry, sharding

    w = geometry.two_bars(L=24, M=14, N=6, xr=(2, 22), zr=(1, 4), y1=(2, 5), y2=(9, 12))
    S, P = problem_of(w)
    freqs = np.array([1e3, 1e7, 5e9])
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        out = sharding.sweep_distributed(freqs, sharding.gpu_sweep_solver(P, tol=1e-12))
    finally:
        dist.destroy_process_group()
    ref = ex.Sweep(P, freqs).prepare().solve(restart=50, tol=1e-12, maxit=10)
    np.testing.assert_array_equal(out["R"], ref["R"])
    np.testing.assert_array_equal(out["L"], ref["L"])
    assert np.all(out["flag"] == 0)


@pytest.mark.parametrize("f", [1e6, 3e9])
def test_precon_schur_gmres_matches_oracle(lib, blob, f):
    """'schur_gmres' (lse_sparse_precon_prepare.m:83-88, lse_sparse_precon_multiply.m:26-46): the inner
    Jacobi-preconditioned GMRES on S takes the oracle's iteration counts and returns its result, for a
    batch mixing frequencies, a zero right-hand side and two inner tolerances."""
    vie, ex = lib
    w, S, P = blob
    fs = [f, 10 * f]
    st = np.stack([1j * 2 * np.pi * fq * solver.MU0 * P.st2 for fq in fs])
    z_real, _ = solver.z_arrays(w.sigma_e, None, 2 * np.pi * f)   # conductors only: z does not depend on f
    g = vie.Geometry(P.fN_all2, S.Ar, z_real, None, S.dx, S.idxS)
    pcs = g.precons(st, kind="schur_gmres")
    pcs[1].set_prectol(1e-3)
    refs = [solver.SparsePrecon("schur_gmres").prepare(S.dx, z_real, None, S.idxS, st[i], S.Ar) for i in range(2)]
    refs[1].prectol = 1e-3
    rng = np.random.default_rng(29)
    X = rng.standard_normal((3, S.n)) + 1j * rng.standard_normal((3, S.n))
    X[2] = 0.0
    batch = [pcs[0], pcs[1], pcs[0]]
    Y = vie.apply_precons(g, batch, X)
    for k, i in enumerate([0, 1, 0]):
        ref = refs[i].multiply(X[k])
        if k == 2:
            assert not np.any(Y[k]) and not np.any(ref)
        else:
            assert rel(Y[k], ref) < 1e-10, k
    assert pcs[0].inner_iterations() == refs[0].inner_iters > 0
    assert pcs[1].inner_iterations() == refs[1].inner_iters > refs[0].inner_iters / 2


def test_fpgmres_schur_gmres_sweep_matches_oracle(lib):
    """The executer's 'schur_gmres' path (flexible outer GMRES, VoxHenry_executer.m:294-297) on two
    bars: converged, with the oracle's outer iterations and R, L."""
    vie, ex = lib
    from voxhenry_gb300 import geometry

    w = geometry.two_bars(L=16, M=10, N=5, xr=(1, 15), zr=(1, 3), y1=(1, 3), y2=(6, 8))
    S, P = problem_of(w)
    freqs = np.array([1e6, 1e9, 2e10])
    sw = ex.Sweep(P, freqs, precon="schur_gmres").prepare()
    out = sw.solve(restart=50, tol=1e-10, maxit=10)
    fN, st = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    ref = solver.solve_frequencies(S, fN, st, freqs, restart=50, tol=1e-10, precon="schur_gmres")
    assert np.all(out["flag"] == 0)
    assert [len(r) - 1 for r in out["resvec"]] == [i[2] for i in ref["iters"]]
    assert_port_matrix_close(out["R"], ref["R"], 1e-8)
    assert_port_matrix_close(out["L"], ref["L"], 1e-8)


def test_mixed_precision_rejects_schur_gmres(lib, blob):
    vie, ex = lib
    w, S, P = blob
    sw = ex.Sweep(P, np.array([1e9]), precon="schur_gmres").prepare()
    with pytest.raises(Exception, match="schur_gmres"):
        sw.solve(restart=20, tol=1e-8, maxit=2, prec="fp32")


def test_factor_sharing_across_frequencies(lib):
    """Sweep.prepare(share_tol): neighbouring frequencies whose A_inv moves by at most share_tol share
    one Schur factor; the sweep still converges and R, L equal the one-factor-per-frequency sweep."""
    vie, ex = lib
    from voxhenry_gb300 import geometry

    w = geometry.two_bars(L=16, M=10, N=5, xr=(1, 15), zr=(1, 3), y1=(1, 3), y2=(6, 8))
    S, P = problem_of(w)
    freqs = np.logspace(3, 10, 12)
    ref = ex.Sweep(P, freqs).prepare().solve(restart=50, tol=1e-10, maxit=10)
    sw = ex.Sweep(P, freqs).prepare(share_tol=1e-6)
    assert 1 < len(np.unique(sw.factor_of)) < len(freqs)
    out = sw.solve(restart=50, tol=1e-10, maxit=10)
    assert np.all(out["flag"] == 0)
    assert_port_matrix_close(out["R"], ref["R"], 1e-8)
    assert_port_matrix_close(out["L"], ref["L"], 1e-8)
    it_ref = np.array([len(r) for r in ref["resvec"]])
    it = np.array([len(r) for r in out["resvec"]])
    assert np.all(it <= it_ref + 1)


def test_serving_alone_and_in_the_mix(lib):
    """Continuous batching (voxhenry_gb300.serving.Server) on small requests of the seeded stream:
    served one at a time on one slot, then all at once on three slots whose work overlaps on the
    device.  Every request converges; each request's R and L in the mix equal its R and L alone within
    1e-6 (the mixed-precision bar); a request for a geometry a slot holds reuses it; and a direct
    FP64 sweep of the first request agrees within 1e-6."""
    import dataclasses

    vie, ex = lib
    from voxhenry_gb300 import serving, structure

    reqs = [r for r in serving.request_stream(80) if r.workload.sigma_e.size < 6e4][:6]
    srv1 = serving.Server(slots=1)
    alone = srv1.run(reqs)
    srv1.close()
    srv3 = serving.Server(slots=3)
    mix = srv3.run(reqs)
    assert srv3.max_in_flight == 3
    for a, m in zip(alone, mix):
        assert a.error is None and m.error is None, (a.error, m.error)
        assert np.all(a.flags == 0) and np.all(m.flags == 0)
        assert_port_matrix_close(m.R, a.R, 1e-6)
        assert_port_matrix_close(m.L, a.L, 1e-6)
    # the same geometry again, with other frequencies: the slot that solved it keeps it resident
    last = mix[-1]
    w_last = reqs[-1].workload
    again = serving.Request(1000, "repeat", dataclasses.replace(w_last, freqs=w_last.freqs[::-1].copy()))
    rec = srv3.run([again])[0]
    assert rec.reused_geometry and rec.slot == last.slot and np.all(rec.flags == 0)
    assert_port_matrix_close(rec.R[::-1], last.R, 1e-6)
    srv3.close()
    w = reqs[0].workload
    P = structure.problem_from_workload(w)
    b = ex.Sweep(P, w.freqs).prepare().solve(restart=50, tol=1e-12, maxit=20)
    assert_port_matrix_close(alone[0].R, b["R"], 1e-6)
    assert_port_matrix_close(alone[0].L, b["L"], 1e-6)


def test_padded_grid_matches_oracle(lib):
    """A 47 x 13 x 5 grid (padded FFT lengths 94, 26 with primes 47, 13) is grown to 48 x 14 x 5 for the
    device FFT; R and L equal the oracle's on the original grid (scipy FFT takes any length)."""
    vie, ex = lib
    from voxhenry_gb300 import geometry
    from voxhenry_gb300 import structure as vstructure

    w = geometry.two_bars(L=47, M=13, N=5, xr=(1, 45), zr=(1, 4), y1=(1, 4), y2=(8, 11))
    P = vstructure.problem_from_workload(w)
    assert P.meta.get("grid_padded_from") == (47, 13, 5)
    freqs = np.array([1e6, 5e9])
    out = ex.Sweep(P, freqs).prepare().solve(restart=50, tol=1e-12, maxit=20)
    fN, st = circulant.generate_circulant_tensor(w.dx, 1.0, 47, 13, 5)
    Sy = solver_system(w)
    ref = solver.solve_frequencies(Sy, fN, st, freqs, restart=50, tol=1e-12)
    assert_port_matrix_close(out["R"], ref["R"], 1e-8)
    assert_port_matrix_close(out["L"], ref["L"], 1e-8)


def solver_system(w):
    return structure.build_system(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght)


def test_two_bars_full_size_known_answer_and_mixed_vs_fp64(lib):
    """The two-bar workload at its full size (128 x 64 x 32, copper and aluminium bars 100 x 10 x 10
    voxels, 2 ports, 16 frequencies 1 kHz-10 GHz): at 1 kHz each bar's resistance is the DC value
    l / (sigma A), and the mixed-precision sweep matches the FP64 sweep (relres < 1e-10) within 1e-6."""
    vie, ex = lib
    from voxhenry_gb300 import geometry
    from voxhenry_gb300 import structure as vstructure

    w = geometry.two_bars()
    P = vstructure.problem_from_workload(w)
    mixed = ex.Sweep(P, w.freqs, precon="schur_invert_df").prepare().solve(restart=50, tol=1e-9, maxit=10,
                                                                           prec="fp32")
    ref = ex.Sweep(P, w.freqs).prepare().solve(restart=50, tol=1e-11, maxit=20)
    assert np.all(mixed["flag"] == 0) and np.all(ref["relres"] < 1e-10)
    for p, sigma in enumerate((5.8e7, 3.5e7)):
        r_dc = 100e-6 / (sigma * (10e-6) ** 2)
        assert abs(ref["R"][0, p, p] - r_dc) <= 1e-6 * r_dc
    for f in range(len(w.freqs)):
        for p in range(2):
            for key in ("R", "L"):
                assert abs(mixed[key][f, p, p] - ref[key][f, p, p]) <= 1e-6 * abs(ref[key][f, p, p])


def test_ring_full_size_mixed_vs_fp64(lib):
    """The ring workload at its full size (512 x 512 x 16, padded FFT grid 1024 x 1024 x 32): at three
    frequencies the mixed-precision R and L match the FP64 sweep (relres < 1e-10) within 1e-6."""
    vie, ex = lib
    from voxhenry_gb300 import geometry
    from voxhenry_gb300 import structure as vstructure

    w = geometry.ring()
    P = vstructure.problem_from_workload(w)
    freqs = w.freqs[[0, 8, 15]]
    mixed = ex.Sweep(P, freqs, precon="schur_invert_df").prepare().solve(restart=50, tol=1e-9, maxit=10,
                                                                         prec="fp32")
    ref = ex.Sweep(P, freqs).prepare().solve(restart=50, tol=1e-11, maxit=20)
    assert np.all(mixed["flag"] == 0) and np.all(ref["relres"] < 1e-10)
    for key in ("R", "L"):
        np.testing.assert_allclose(mixed[key], ref[key], rtol=1e-6)


def superconducting_bar():
    """A bar whose first half is a superconductor (London depth 0.1 um, normal-fluid sigma as the
    copper), so that z is complex and depends on omega (VoxHenry_executer.m:236-259)."""
    from voxhenry_gb300 import geometry

    w = geometry.bar(L=16, M=5, N=4, dx=0.5e-6)
    lam = np.zeros(w.sigma_e.shape, order="F")
    lam[:8] = 1e-7
    w.lambdaL = lam
    return w


@pytest.mark.parametrize("f", [1e6, 2e10])
def test_precon_superconductor_matches_oracle(lib, f):
    """lse_sparse_precon_prepare's z_real + z_imag branch (prepare.m:42-46) on the device."""
    vie, ex = lib
    w = superconducting_bar()
    S, P = problem_of(w)
    om = 2 * np.pi * f
    jwmu = 1j * om * solver.MU0
    z_real, z_imag = solver.z_arrays(w.sigma_e, w.lambdaL, om)
    assert np.abs(z_imag).max() > 0
    ref = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, z_imag, S.idxS, jwmu * P.st2, S.Ar)
    g = vie.Geometry(P.fN_all2, S.Ar, z_real, z_imag, S.dx, S.idxS)
    pc = g.precon(jwmu * P.st2)
    X = np.random.default_rng(31).standard_normal((2, S.n)) + 1j * np.random.default_rng(32).standard_normal((2, S.n))
    Y = vie.apply_precons(g, [pc, pc], X)
    for k in range(2):
        assert rel(Y[k], ref.multiply(X[k])) < PRECON_TOL


def test_superconductor_sweep_matches_oracle(lib):
    """A sweep with one omega-dependent z slot per frequency (VoxHenry_executer.m:236-259) through the
    factor, the FFT matvec and GMRES: FP64 R, L and x within 1e-9 of the oracle at 100 MHz and 20 GHz,
    mixed precision within 1e-6.  At 1 kHz the superconducting half is a near-short (|z| ~ 1e-8 of
    copper's), A_inv spans ten decades and the oracle's own true relative residual stops at ~1e-5 even
    at GMRES tol 1e-14: there any change of rounding (two exact factorisations of S, two FFTs) moves the
    solution by up to that floor, and R, L are compared to 1e-4."""
    vie, ex = lib
    w = superconducting_bar()
    S, P = problem_of(w)
    freqs = np.array([1e3, 1e8, 2e10])
    ref = solver.solve_frequencies(S, P.fN_all2, P.st2, freqs, restart=50, tol=1e-12, keep_x=True)
    sw = ex.Sweep(P, freqs)
    assert sw.super and list(sw.zslot) == [0, 1, 2]
    out = sw.prepare().solve(restart=50, tol=1e-12, maxit=10)
    for k, bound in enumerate((1e-4, 1e-9, 1e-9)):
        assert_port_matrix_close(out["R"][k:k + 1], ref["R"][k:k + 1], bound)
        assert_port_matrix_close(out["L"][k:k + 1], ref["L"][k:k + 1], bound)
    for k in (1, 2):
        assert rel(out["x"][k], ref["x"][k]) < 1e-9
    # mixed precision refines on the true residual, which the 1 kHz near-short cannot bring to 1e-10
    swm = ex.Sweep(P, freqs[1:], precon="schur_invert_df")
    outm = swm.prepare().solve(restart=50, tol=1e-10, maxit=10, prec="fp32")
    assert np.all(outm["flag"] == 0)
    assert_port_matrix_close(outm["R"], ref["R"][1:], 1e-6)
    assert_port_matrix_close(outm["L"], ref["L"][1:], 1e-6)
    for k in range(2):
        assert rel(outm["x"][k], ref["x"][k + 1]) < 1e-6


def test_pgmres_initial_guess_and_right_preconditioner(lib, blob):
    """pgmres(A, b, restart, tol, maxit, L1, [], [], [], x0) and pgmres(..., [], [], R1) (pgmres.m:70)
    against the oracle's pgmres with the same arguments; the mixed solver refines from x0 too."""
    vie, ex = lib
    w, S, P = blob
    f = 2.5e9
    om = 2 * np.pi * f
    jwmu = 1j * om * solver.MU0
    fN = jwmu * P.fN_all2
    st = jwmu * P.st2
    z_real, z_imag = solver.z_arrays(w.sigma_e, None, om)
    ref = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, z_imag, S.idxS, st, S.Ar)
    vie.lse_sparse_precon_prepare(S.dx, z_real, z_imag, S.idxS, st, S.nodeid_4_grnd, S.nodeid_4_injectcurr, S.Ar)
    A = vie.matvec_handle(fN, S.Ar, z_real, z_imag, S.dx, S.idxS5)
    Aref = lambda J: solver.lse_matvect_mult(J, fN, S.Ar, z_real, z_imag, S.dx, S.idxS5)
    b = S.rhs[:, 0].astype(complex)
    rng = np.random.default_rng(41)
    x0 = 1e-3 * (rng.standard_normal(S.n) + 1j * rng.standard_normal(S.n))
    xg, flag, relres, it, resvec = vie.pgmres(A, b, 100, 1e-12, 10, vie.precon_handle(), x0=x0)
    xo, flag_o, relres_o, it_o, resvec_o = solver.pgmres(Aref, b, 100, 1e-12, 10, ref.multiply, x0=x0)
    assert rel(xg, xo) < 1e-9
    np.testing.assert_allclose(resvec[0], resvec_o[0], rtol=1e-9)   # |M^-1 (b - A x0)| / |M^-1 b|
    assert flag == flag_o and relres < 1e-10
    # right preconditioning (R1): the flexible solver with a fixed preconditioner
    xr, flag_r, relres_r, it_r, resvec_r = vie.pgmres(A, b, 100, 1e-11, 10, None, None, vie.precon_handle())
    xor, *_ = solver.pgmres(Aref, b, 100, 1e-11, 10, None, ref.multiply)
    assert rel(xr, xor) < 1e-9 and flag_r == 0
    # the mixed-precision solver from x0 (a geometry with the complex64 tensor, the batched form)
    g = vie.Geometry(P.fN_all2, S.Ar, z_real, None, S.dx, S.idxS, want_fp32=True)
    pc = g.precon(st, kind="schur_invert_df")
    out = g.solve(b[None], pcs=[pc], scale=jwmu, restart=50, tol=1e-10, maxit=10, prec="fp32", x0=x0[None])
    assert out["flag"][0] == 0 and out["relres"][0] <= 1e-10
    assert rel(out["x"][0], xo) < 1e-8
    with pytest.raises(NotImplementedError):
        vie.pgmres(A, b, 100, 1e-12, 10, vie.precon_handle(), None, vie.precon_handle())
