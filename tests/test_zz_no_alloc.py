"""vh_matvec_device_noalloc (allocation-free FFT matvec) vs vh_matvec_device, through the C ABI.

The allocation-free entry point serves callers that cannot allocate device memory at call time; it
must give the results of the regular entry point on consecutive calls.  Collected last so that it
also runs after everything else has used the device.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12     # single FP64 matvec, relative 2-norm
FP32_TOL = 2e-6      # complex64 FFT convolution, relative 2-norm
SCRATCH_BYTES = 16 << 20
VH_ERR_BAD_ARG = 1
VH_ERR_UNSUPPORTED = 3


@pytest.fixture(scope="module")
def env():
    import __graft_entry__

    __graft_entry__.build()
    import torch

    from voxhenry_gb300 import _lib, executer, geometry, structure, vie

    return torch, _lib, executer, geometry, structure, vie


def make_geometry(env, w, want_fp32=True):
    torch, _lib, executer, geometry, structure, vie = env
    prob = structure.problem_from_workload(w)
    z_real, z_imag = executer.z_arrays(w.sigma_e, w.lambdaL, 2 * np.pi * 1e9)
    g, _ = vie.Geometry.generated(prob.L, prob.M, prob.N, prob.dx, prob.Ar, z_real, z_imag, prob.idxS,
                                  want_fp32=want_fp32)
    return g, z_real


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def run(env, fn, g, X, scale, zslot, prec):
    """Calls `fn` (a C ABI matvec with device pointers) on B RHS; returns (status, host result)."""
    torch, _lib = env[0], env[1]
    B = X.shape[0]
    x = torch.from_numpy(np.ascontiguousarray(X).view(np.float64)).cuda()
    y = torch.full_like(x, float("nan"))
    s = None if scale is None else torch.from_numpy(np.ascontiguousarray(scale).view(np.float64)).cuda()
    zs = None if zslot is None else np.ascontiguousarray(zslot, dtype=np.int32)
    st = fn(g.handle, B, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
            None if s is None else C.c_void_p(s.data_ptr()),
            None if zs is None else zs.ctypes.data_as(C.POINTER(C.c_int)), _lib.PREC[prec])
    g.ctx.synchronize()
    return st, y.cpu().numpy().view(np.complex128).reshape(B, g.n)


def check_twice(env, g, X, scale, zslot, prec, tol):
    lib = g.ctx._lib
    st, ref = run(env, lib.vh_matvec_device, g, X, scale, zslot, prec)
    env[1].check(st, g.ctx.handle)
    for _ in range(2):    # two calls in a row: the fixed scratch is reused as left by the first
        st, got = run(env, lib.vh_matvec_device_noalloc, g, X, scale, zslot, prec)
        env[1].check(st, g.ctx.handle)
        assert np.all(np.isfinite(got))
        for b in range(X.shape[0]):
            assert rel(got[b], ref[b]) < tol


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL)])
def test_noalloc_matches_matvec_device(env, prec, tol):
    geometry = env[3]
    g, _ = make_geometry(env, geometry.random_blob((10, 7, 6), fill=0.6, seed=11))
    rng = np.random.default_rng(5)
    X = rng.standard_normal((3, g.n)) + 1j * rng.standard_normal((3, g.n))
    scale = 1j * 2 * np.pi * np.array([1e3, 1e8, 2e10]) * 4e-7 * np.pi
    check_twice(env, g, X, scale, None, prec, tol)
    check_twice(env, g, X, None, None, prec, tol)       # unit scale (the drop-in form)


def test_noalloc_groups_by_slot_and_scratch(env):
    """12 RHS on a 24 x 14 x 10 grid need two scratch groups in FP64; mixed z slots split them further."""
    geometry = env[3]
    g, z_real = make_geometry(env, geometry.random_blob((24, 14, 10), fill=0.7, seed=4))
    g.set_z(1, z_real * 1.9)
    per_rhs = 30 * 24 * 14 * 10 * 16
    assert 12 * per_rhs > SCRATCH_BYTES > per_rhs
    rng = np.random.default_rng(8)
    B = 12
    X = rng.standard_normal((B, g.n)) + 1j * rng.standard_normal((B, g.n))
    scale = 1j * 2 * np.pi * np.logspace(3, 10, B) * 4e-7 * np.pi
    check_twice(env, g, X, scale, None, "fp64", FP64_TOL)
    zslot = [0, 0, 1, 1, 1, 0, 0, 0, 1, 0, 1, 1]
    check_twice(env, g, X, scale, zslot, "fp64", FP64_TOL)
    check_twice(env, g, X, scale, zslot, "fp32", FP32_TOL)


def test_noalloc_rejects_grid_beyond_scratch(env):
    """36 x 32 x 32: one FP64 RHS needs 17.7 MB of FFT scratch (> 16 MiB) -> VH_ERR_UNSUPPORTED; FP32 fits."""
    geometry = env[3]
    g, _ = make_geometry(env, geometry.bar(L=36, M=32, N=32, dx=1e-6))
    lib = g.ctx._lib
    rng = np.random.default_rng(9)
    X = rng.standard_normal((2, g.n)) + 1j * rng.standard_normal((2, g.n))
    st, _ = run(env, lib.vh_matvec_device_noalloc, g, X, None, None, "fp64")
    assert st == VH_ERR_UNSUPPORTED
    assert b"scratch" in lib.vh_last_error(g.ctx.handle)
    check_twice(env, g, X, None, None, "fp32", FP32_TOL)


def test_noalloc_matches_the_oracle(env):
    """FP64 allocation-free products against the oracle's lse_matvect_mult (lse_matvect_mult.m:1-140)
    on the same geometry: the oracle's own circulant tensor, panel numbering and Ae."""
    from oracle import circulant, solver, structure

    geometry, vie = env[3], env[5]
    w = geometry.random_blob((9, 6, 5), fill=0.65, seed=21)
    S = structure.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    fN, _ = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    z_real, _ = solver.z_arrays(w.sigma_e, None, 2 * np.pi * 1e9)
    g = vie.Geometry(fN, S.Ar, z_real, None, S.dx, S.idxS)
    rng = np.random.default_rng(23)
    X = rng.standard_normal((2, S.n)) + 1j * rng.standard_normal((2, S.n))
    jwmu = 1j * 2 * np.pi * np.array([1e6, 2e10]) * solver.MU0
    for _ in range(2):
        st, got = run(env, g.ctx._lib.vh_matvec_device_noalloc, g, X, jwmu, None, "fp64")
        env[1].check(st, g.ctx.handle)
        for b in range(2):
            ref = solver.lse_matvect_mult(X[b], jwmu[b] * fN, S.Ar, z_real, None, S.dx, S.idxS5)
            assert rel(got[b], ref) < FP64_TOL


def test_noalloc_allocates_nothing_on_a_new_geometry(env):
    """The first product on a fresh geometry, before any regular product could size its scratch, leaves
    the device's free memory unchanged (the regular path would grow ~30 L M N complex values per RHS)."""
    torch, geometry = env[0], env[3]
    # a geometry of the same shape first: loads the kernels these grids use (lazy module loading takes
    # device memory for code) and sets up the fixed arrays
    warm, _ = make_geometry(env, geometry.random_blob((30, 20, 12), fill=0.6, seed=2))
    rng = np.random.default_rng(4)
    Xw = rng.standard_normal((2, warm.n)) + 1j * rng.standard_normal((2, warm.n))
    for prec in ("fp64", "fp32"):
        env[1].check(run(env, warm.ctx._lib.vh_matvec_device_noalloc, warm, Xw, None, None, prec)[0], warm.ctx.handle)
    g, _ = make_geometry(env, geometry.random_blob((30, 20, 12), fill=0.6, seed=3))
    lib = g.ctx._lib
    B = 6
    X = rng.standard_normal((B, g.n)) + 1j * rng.standard_normal((B, g.n))
    x = torch.from_numpy(np.ascontiguousarray(X).view(np.float64)).cuda()
    y = torch.empty_like(x)
    for prec in ("fp64", "fp32"):
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        st = lib.vh_matvec_device_noalloc(g.handle, B, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), None, None,
                                          env[1].PREC[prec])
        g.ctx.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        env[1].check(st, g.ctx.handle)
        assert free1 == free0, (prec, free0 - free1)
        assert np.all(np.isfinite(y.cpu().numpy()))


def test_noalloc_rejects_double_float(env):
    """VH_PREC_DF builds a pair copy of the tensor (an allocation): VH_ERR_BAD_ARG."""
    geometry = env[3]
    g, _ = make_geometry(env, geometry.random_blob((8, 6, 5), fill=0.6, seed=6))
    X = np.ones((1, g.n), dtype=np.complex128)
    st, _ = run(env, g.ctx._lib.vh_matvec_device_noalloc, g, X, None, None, "df")
    assert st == VH_ERR_BAD_ARG
