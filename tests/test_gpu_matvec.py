"""FFT matvec parity: GPU (through the C ABI) vs the CPU oracle's lse_matvect_mult."""
import numpy as np
import pytest

from conftest import golden_vhr_text
from oracle import circulant, solver, structure, vhr

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12     # single FP64 matvec, relative 2-norm
FP32_TOL = 2e-6      # complex64 FFT convolution, relative 2-norm
DF_TOL = 1e-12       # double-float passes (~48 significant bits), relative 2-norm


@pytest.fixture(scope="module")
def vie():
    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import vie as v

    return v


def system_of(w):
    S = structure.build_system(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght)
    fN, st = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    return S, fN, st


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def rand_c(rng, n):
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


GRIDS = [(2, 4, 4), (6, 5, 4), (5, 7, 3), (12, 10, 9), (16, 8, 8), (20, 6, 5)]


@pytest.mark.parametrize("shape", GRIDS)
def test_matvec_fp64_random_grids(vie, shape):
    from voxhenry_gb300 import geometry

    w = geometry.random_blob(shape, fill=0.65, seed=sum(shape))
    S, fN, st = system_of(w)
    f = 2.5e9
    jwmu = 1j * 2 * np.pi * f * solver.MU0
    fNf = jwmu * fN
    z_real, _ = solver.z_arrays(w.sigma_e, None, 2 * np.pi * f)
    rng = np.random.default_rng(3)
    x = rand_c(rng, S.n)
    ref = solver.lse_matvect_mult(x, fNf, S.Ar, z_real, None, S.dx, S.idxS5)
    got = vie.lse_matvect_mult(x, fNf, S.Ar, z_real, None, S.dx, S.idxS5)
    assert rel(got, ref) < FP64_TOL


def test_matvec_numex1_reference_input(vie):
    """The reference's own numex1 input (60 x 20 x 20, padded 120 x 40 x 40: radices 2, 3, 5)."""
    inp = vhr.read_vhr_text(golden_vhr_text("straight_cond1_len30.0u_wid10.0u_dist20.0u.vhr"))
    S = structure.build_system(inp.sigma_e, None, inp.dx, inp.pnt_lft, inp.pnt_rght)
    fN, st = circulant.generate_circulant_tensor(inp.dx, 1.0, S.L, S.M, S.N)
    f = 1e10
    fNf = (1j * 2 * np.pi * f * solver.MU0) * fN
    z_real, _ = solver.z_arrays(inp.sigma_e, None, 2 * np.pi * f)
    rng = np.random.default_rng(5)
    for _ in range(2):
        x = rand_c(rng, S.n)
        ref = solver.lse_matvect_mult(x, fNf, S.Ar, z_real, None, S.dx, S.idxS5)
        got = vie.lse_matvect_mult(x, fNf, S.Ar, z_real, None, S.dx, S.idxS5)
        assert rel(got, ref) < FP64_TOL


def test_matvec_superconductor(vie):
    """z_imag present (two-fluid superconductor, VoxHenry_executer.m:236-259)."""
    from voxhenry_gb300 import geometry

    w = geometry.random_blob((8, 6, 5), fill=0.7, seed=11)
    lam = np.where(w.sigma_e > 0, 5e-8, 0.0)
    w.lambdaL = np.asfortranarray(lam)
    S, fN, st = system_of(w)
    f = 5e9
    om = 2 * np.pi * f
    z_real, z_imag = solver.z_arrays(w.sigma_e, w.lambdaL, om)
    fNf = (1j * om * solver.MU0) * fN
    x = rand_c(np.random.default_rng(9), S.n)
    ref = solver.lse_matvect_mult(x, fNf, S.Ar, z_real, z_imag, S.dx, S.idxS5)
    got = vie.lse_matvect_mult(x, fNf, S.Ar, z_real, z_imag, S.dx, S.idxS5)
    assert rel(got, ref) < FP64_TOL


def test_matvec_batched_scales_and_slots(vie):
    """B right-hand sides with per-RHS j*omega*mu and per-RHS z: each equals its single-RHS product."""
    from voxhenry_gb300 import geometry

    w = geometry.random_blob((10, 8, 6), fill=0.6, seed=21)
    S, fN, st = system_of(w)
    z_real, _ = solver.z_arrays(w.sigma_e, None, 1.0)
    g = vie.Geometry(fN, S.Ar, z_real, None, S.dx, S.idxS, want_fp32=True)
    z2 = z_real * 1.7
    g.set_z(1, z2)
    freqs = np.array([1e3, 1e6, 1e9, 2e10])
    scales = 1j * 2 * np.pi * freqs * solver.MU0
    slots = np.array([0, 1, 0, 1], dtype=np.int32)
    rng = np.random.default_rng(2)
    X = np.stack([rand_c(rng, S.n) for _ in freqs])
    Yb = g.matvec(X, scale=scales, zslot=slots)
    for b in range(len(freqs)):
        zr = z_real if slots[b] == 0 else z2
        ref = solver.lse_matvect_mult(X[b], scales[b] * fN, S.Ar, zr, None, S.dx, S.idxS5)
        assert rel(Yb[b], ref) < FP64_TOL
        single = g.matvec(X[b], scale=scales[b], zslot=int(slots[b]))
        assert np.array_equal(single, Yb[b])      # batching invariance: bitwise
    Y32 = g.matvec(X, scale=scales, zslot=slots, prec="fp32")
    for b in range(len(freqs)):
        assert rel(Y32[b], Yb[b]) < FP32_TOL


def test_matvec_linearity_large(vie):
    """Size-independent property on the full 64 x 16 x 16 bar workload: A(ax + by) = aAx + bAy."""
    from voxhenry_gb300 import geometry

    w = geometry.bar()
    S = structure.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    fN, st = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    z_real, _ = solver.z_arrays(w.sigma_e, None, 1.0)
    g = vie.Geometry(fN, S.Ar, z_real, None, S.dx, S.idxS)
    rng = np.random.default_rng(4)
    x, y = rand_c(rng, S.n), rand_c(rng, S.n)
    a, b = 0.3 - 1.1j, 2.0 + 0.5j
    s = 1j * 2 * np.pi * 1e9 * solver.MU0
    lhs = g.matvec(a * x + b * y, scale=s)
    rhs = a * g.matvec(x, scale=s) + b * g.matvec(y, scale=s)
    assert rel(lhs, rhs) < 1e-13
    ref = solver.lse_matvect_mult(x, s * fN, S.Ar, z_real, None, S.dx, S.idxS5)
    assert rel(g.matvec(x, scale=s), ref) < FP64_TOL


BOXES = [  # (grid, z range): padded z lengths 18 (shared-memory z-pass) and 8, 16, 32 (register z-pass)
    ((20, 16, 9), (2, 6)),
    ((16, 10, 4), (1, 2)),
    ((20, 16, 8), (2, 5)),
    ((12, 10, 16), (3, 8)),
    ((12, 10, 16), (0, 16)),
]


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL), ("df", DF_TOL)])
@pytest.mark.parametrize("shape,zr", BOXES)
def test_matvec_voxel_box_inside_grid(vie, prec, tol, shape, zr):
    """Voxels in a y and z sub-range of the grid: the transform visits only that box."""
    from voxhenry_gb300 import geometry

    L, M, N = shape
    w = geometry.two_bars(L=L, M=M, N=N, xr=(1, L - 1), zr=zr, y1=(1, 3), y2=(M - 4, M - 1))
    S, fN, st = system_of(w)
    z_real, _ = solver.z_arrays(w.sigma_e, None, 1.0)
    g = vie.Geometry(fN, S.Ar, z_real, None, S.dx, S.idxS, want_fp32=True)
    s = 1j * 2 * np.pi * 3e9 * solver.MU0
    rng = np.random.default_rng(12)
    X = np.stack([rand_c(rng, S.n) for _ in range(3)])
    Y = g.matvec(X, scale=np.full(3, s), prec=prec)
    for b in range(3):
        ref = solver.lse_matvect_mult(X[b], s * fN, S.Ar, z_real, None, S.dx, S.idxS5)
        assert rel(Y[b], ref) < tol


DF_BOXES = BOXES + [  # padded x and y lengths 256 (the double-float passes' shapes), z 8 / 16 / 18
    ((128, 128, 4), (1, 3)),
    ((128, 128, 8), (2, 5)),
    ((128, 128, 9), (2, 6)),
]


@pytest.mark.parametrize("shape,zr", DF_BOXES)
def test_matvec_df_takes_the_double_float_passes(vie, shape, zr):
    """VH_PREC_DF differs from FP64 only by double-float rounding where the double-float passes run
    (padded x and y lengths 256, 512 or 1024 and z length 8, 16 or 32), and equals FP64 bit for bit
    where it falls back to the complex128 product."""
    from voxhenry_gb300 import geometry

    L, M, N = shape
    w = geometry.two_bars(L=L, M=M, N=N, xr=(1, L - 1), zr=zr, y1=(1, 3), y2=(M - 4, M - 1))
    S, fN, st = system_of(w)
    z_real, _ = solver.z_arrays(w.sigma_e, None, 1.0)
    g = vie.Geometry(fN, S.Ar, z_real, None, S.dx, S.idxS)
    rng = np.random.default_rng(5)
    X = np.stack([rand_c(rng, S.n) for _ in range(2)])
    s = np.full(2, 1j * 2 * np.pi * 3e9 * solver.MU0)   # j omega mu: the convolution carries the product
    Y64 = g.matvec(X, scale=s, prec="fp64")
    Ydf = g.matvec(X, scale=s, prec="df")
    d = max(rel(Ydf[b], Y64[b]) for b in range(2))
    if 2 * L in (256, 512, 1024) and 2 * M in (256, 512, 1024) and 2 * N in (8, 16, 32):
        assert 0 < d < DF_TOL
        ref = solver.lse_matvect_mult(X[0], s[0] * fN, S.Ar, z_real, None, S.dx, S.idxS5)
        assert rel(Ydf[0], ref) < DF_TOL   # and against the oracle
    else:
        assert d == 0


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL), ("df", DF_TOL)])
def test_every_tuning_choice_gives_the_product(vie, prec, tol):
    """Each launch choice the autotuner can make (vh_conv_set_tuning: the register y-pass over 128- or
    64-byte row segments or the Stockham y-pass, the two-lane or the one-thread-per-column z-pass or (complex64) the direct Toeplitz z
    convolution, the shared-memory or (complex64) warp-per-line x passes, the whole batch or chunks of 4
    right-hand sides) gives the FP64 product of the
    default within the precision's tolerance; vh_conv_tune picks one of them and leaves it set.
    A variant a precision does not take (z 3 in FP64) falls back to the automatic pass."""
    import ctypes as C

    from voxhenry_gb300 import _lib, executer, geometry, structure

    w = geometry.random_blob((128, 128, 4), fill=0.2, seed=9)    # padded 256 x 256 x 8: both y-passes apply
    prob = structure.problem_from_workload(w)
    z_real, _ = executer.z_arrays(w.sigma_e, None, 2 * np.pi * 1e9)
    g, _ = vie.Geometry.generated(prob.L, prob.M, prob.N, prob.dx, prob.Ar, z_real, None, prob.idxS, want_fp32=True)
    rng = np.random.default_rng(21)
    B = 6
    X = np.stack([rand_c(rng, g.n) for _ in range(B)])
    scale = 1j * 2 * np.pi * np.logspace(6, 10, B) * solver.MU0
    ref = g.matvec(X, scale=scale, prec="fp64")
    lib = g.ctx._lib
    for yv in (1, 2, 3):
        for zv in (1, 2, 3):
            for mr in (0, 4):
                for xv in ((0, 1, 2) if prec == "fp32" else (0,)):
                    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC[prec], yv, zv, mr, xv), g.ctx.handle)
                    got = g.matvec(X, scale=scale, prec=prec)
                    for b in range(B):
                        assert rel(got[b], ref[b]) < tol, (yv, zv, mr, xv, b)
    yv, zv, mr, xv, ms = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_double()
    _lib.check(lib.vh_conv_tune(g.handle, _lib.PREC[prec], B, C.byref(yv), C.byref(zv), C.byref(mr), C.byref(xv),
                                C.byref(ms)), g.ctx.handle)
    assert yv.value in (1, 2, 3) and zv.value in ((1, 2) if prec == "fp64" else (1, 2, 3)) and mr.value in (0, 4)
    assert ms.value > 0 and xv.value in ((1, 2) if prec == "fp32" else (0,))
    got = g.matvec(X, scale=scale, prec=prec)
    assert max(rel(got[b], ref[b]) for b in range(B)) < tol
    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC[prec], 0, 0, 0, 0), g.ctx.handle)


@pytest.mark.parametrize("shape,fill", [((40, 24, 7), 0.3), ((16, 16, 16), 0.9), ((30, 20, 3), 0.5),
                                        ((64, 32, 10), 0.4)])
def test_toeplitz_z_pass_matches_the_fft_product(vie, shape, fill):
    """The direct z convolution (z_variant 3, complex64) against the oracle's FP64 product, over box
    heights 3 to 16 (odd heights run with one zero row of padding) and a padded x length (80) that is
    not a multiple of the kernel's 32 columns.  Its product is not bitwise the
    FFT z-pass's (a different kernel ran) but within the same complex64 tolerance."""
    from voxhenry_gb300 import _lib, executer, geometry

    w = geometry.random_blob(shape, fill=fill, seed=31)
    S = structure.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    fN, _ = circulant.generate_circulant_tensor(S.dx, 1.0, S.L, S.M, S.N)
    z_real, _ = solver.z_arrays(w.sigma_e, None, 1.0)
    g = vie.Geometry(fN, S.Ar, z_real, None, S.dx, S.idxS, want_fp32=True)
    rng = np.random.default_rng(5)
    B = 3
    X = np.stack([rand_c(rng, g.n) for _ in range(B)])
    scale = 1j * 2 * np.pi * np.array([1e6, 1e9, 2e10]) * solver.MU0
    lib = g.ctx._lib
    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC["fp32"], 0, 1, 0, 0), g.ctx.handle)
    fft = g.matvec(X, scale=scale, prec="fp32")
    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC["fp32"], 0, 3, 0, 0), g.ctx.handle)
    toep = g.matvec(X, scale=scale, prec="fp32")
    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC["fp32"], 0, 0, 0, 0), g.ctx.handle)
    assert not np.array_equal(fft, toep)
    for b in range(B):
        ref = solver.lse_matvect_mult(X[b], scale[b] * fN, S.Ar, z_real, None, S.dx, S.idxS5)
        assert rel(toep[b], ref) < FP32_TOL, b
        assert rel(fft[b], ref) < FP32_TOL, b


@pytest.mark.parametrize("shape,height", [((128, 128, 4), 4), ((128, 128, 8), 8), ((128, 128, 16), 16),
                                          ((128, 128, 16), 7), ((128, 128, 16), 10)])
def test_toeplitz_z_pass_double_float(vie, shape, height):
    """The direct z convolution in double-float arithmetic (z_variant 3 of VH_PREC_DF) on grids the
    double-float product takes (padded 256 x 256 x 8, 16, 32) with voxel-box heights 4, 8, 16 and, on
    the tallest grid with the upper layers empty, 7 (an odd height: one zero row of padding) and 10:
    within the double-float tolerance of the oracle's FP64 product, and not bitwise the FFT z-pass's."""
    from voxhenry_gb300 import _lib, geometry

    w = geometry.random_blob(shape, fill=0.1, seed=17)
    sigma = np.array(w.sigma_e)
    sigma[:, :, height:] = 0.0
    m1 = np.zeros(shape, bool)
    m1[0, :, :height] = True
    m2 = np.zeros(shape, bool)
    m2[-1, :, :height] = True
    S = structure.build_system(np.asfortranarray(sigma), None, w.dx, [geometry.face_nodes(m1, "-x")],
                               [geometry.face_nodes(m2, "+x")])
    fN, _ = circulant.generate_circulant_tensor(S.dx, 1.0, S.L, S.M, S.N)
    z_real, _ = solver.z_arrays(np.asfortranarray(sigma), None, 1.0)
    g = vie.Geometry(fN, S.Ar, z_real, None, S.dx, S.idxS, want_fp32=True)
    rng = np.random.default_rng(8)
    B = 3
    X = np.stack([rand_c(rng, g.n) for _ in range(B)])
    scale = 1j * 2 * np.pi * np.array([1e6, 1e9, 2e10]) * solver.MU0
    lib = g.ctx._lib
    fft = g.matvec(X, scale=scale, prec="df")
    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC["df"], 0, 3, 0, 0), g.ctx.handle)
    toep = g.matvec(X, scale=scale, prec="df")
    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC["df"], 0, 0, 0, 0), g.ctx.handle)
    assert not np.array_equal(fft, toep)
    for b in range(B):
        ref = solver.lse_matvect_mult(X[b], scale[b] * fN, S.Ar, z_real, None, S.dx, S.idxS5)
        assert rel(toep[b], ref) < DF_TOL, b
        assert rel(fft[b], ref) < DF_TOL, b


@pytest.mark.parametrize("shape", [(128, 40, 6), (256, 24, 4), (512, 12, 2)])
def test_warp_x_passes_match_the_product(vie, shape):
    """The warp-per-line x passes (x variant 1, complex64) on padded x lengths 256, 512 and 1024 against
    the oracle's FP64 product, and not bitwise the shared-memory passes' product."""
    from voxhenry_gb300 import _lib, geometry

    w = geometry.random_blob(shape, fill=0.3, seed=23)
    S = structure.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    fN, _ = circulant.generate_circulant_tensor(S.dx, 1.0, S.L, S.M, S.N)
    z_real, _ = solver.z_arrays(w.sigma_e, None, 1.0)
    g = vie.Geometry(fN, S.Ar, z_real, None, S.dx, S.idxS, want_fp32=True)
    rng = np.random.default_rng(6)
    B = 3
    X = np.stack([rand_c(rng, g.n) for _ in range(B)])
    scale = 1j * 2 * np.pi * np.array([1e6, 1e9, 2e10]) * solver.MU0
    lib = g.ctx._lib
    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC["fp32"], 0, 0, 0, 2), g.ctx.handle)
    smem = g.matvec(X, scale=scale, prec="fp32")
    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC["fp32"], 0, 0, 0, 1), g.ctx.handle)
    warp = g.matvec(X, scale=scale, prec="fp32")
    _lib.check(lib.vh_conv_set_tuning(g.handle, _lib.PREC["fp32"], 0, 0, 0, 0), g.ctx.handle)
    assert not np.array_equal(smem, warp)
    for b in range(B):
        ref = solver.lse_matvect_mult(X[b], scale[b] * fN, S.Ar, z_real, None, S.dx, S.idxS5)
        assert rel(warp[b], ref) < FP32_TOL, b

