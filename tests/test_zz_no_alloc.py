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
