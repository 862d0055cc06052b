"""GPU parity on the four benchmark configurations against the oracle's committed fixtures.

The oracle (the FP64 restatement of the reference path) solved each configuration's seeded
synthetic workload to GMRES tol 1e-14, and once more to 1e-12 to measure how much each point's
R, L and x are left undetermined by its conditioning (tests/golden/make_config_fixtures.py).  Here
the GPU solves the same frequencies through the batched sweep (executer.Sweep -> vh_gmres) and is
held to:
  * the plain FP64 path at the fixtures' tol 1e-14: R, L and the current density x within 1e-9 or,
    where a point is more sensitive, within 10 times the oracle's own change between its two solves
    (the spiral's 20 GHz resistance moves by 1.1e-8 between them, a small real part of a mostly
    inductive impedance, and its x by up to 6e-9) or twice the point's sensitivity to the rounding
    noise of the tensor spectrum: the change of R, L between this FP64 solve (the complex spectrum)
    and a converged solve of the mixed path (tol 1e-12, the real/imaginary form of the same spectrum,
    which drops its ~1e-12 rounding noise).  Both solves end at their FP64 floor; at the ring's
    20 GHz point they differ by 1.2e-8 in R, and so does every FP64 computation of the tensor (the
    oracle's included), the spiral's by 6e-8, while the other points move by less than 1e-10;
  * the mixed-precision path (complex64 FFT matvec inside FP64 refinement, double-float Schur
    factor) at the benchmark's tol 1e-10: R, L and x within 1e-6;
  * the straight bar at its own settings (tol 1e-8, restart 50, maxit 10): the oracle's iteration
    counts, R and L within 1e-9 of the oracle's at the same settings, and x within 1e-8 (both
    iterates stop at the same step short of convergence, where rounding differences of the two
    implementations -- their Schur factors, FFTs and sums -- are amplified to a few 1e-9).
R and L are compared per frequency relative to the largest entry of the port matrix (the mutual
terms of the decoupled two bars sit near the rounding floor of the self terms).  x is compared
norm-wise through a 64-row Gaussian sketch (which estimates |x - x_ref| / |x_ref| within about
25 %) and element-wise on a strided sample.
"""
import os

import numpy as np
import pytest

import config_fixtures as cf

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-9        # plain FP64 GPU path against the oracle
MIXED_TOL = 1e-6       # mixed-precision path against the oracle
OWN_SETTINGS_X_TOL = 1e-8   # x of two unconverged iterates (tol 1e-8) of the same algorithm
NAMES = list(cf.CONFIGS)


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import executer, geometry, structure

    return executer, geometry, structure


_SWEEPS = {}


def sweep_of(lib, name):
    """The GPU sweep of the fixture's frequencies of one configuration (built once per module)."""
    executer, geometry, structure = lib
    if name not in _SWEEPS:
        for k in list(_SWEEPS):          # one configuration resident at a time (the ring takes ~7 GB)
            _SWEEPS.pop(k)[1].geom.close()
        if not os.path.exists(cf.path(name)):
            pytest.skip(f"fixture {cf.path(name)} not generated")
        fx = cf.load(name)
        w = geometry.WORKLOADS[name]()
        prob = structure.problem_from_workload(w)
        sw = executer.Sweep(prob, fx["freqs"], want_fp32=True)
        assert sw.geom.n == int(fx["n"]) and prob.Ar.shape[1] == int(fx["nc"])
        _SWEEPS[name] = (fx, sw)
    return _SWEEPS[name]


def rel_port(a, b):
    return np.array([np.abs(a[k] - b[k]).max() / np.abs(b[k]).max() for k in range(b.shape[0])])


def check_x(out, fx, nc, bound, prefix="x_"):
    d = cf.compare(out["x"], nc, fx, prefix)
    assert d["curr_sketch"] < bound, d
    assert d["phi_sketch"] < bound, d
    assert d["curr_sample"] < 10 * bound, d
    assert d["curr_norm"] < bound, d
    return d


@pytest.mark.parametrize("name", NAMES)
def test_fp64_matches_oracle(lib, name):
    fx, sw = sweep_of(lib, name)
    sw.precon_kind = "schur_invert"
    sw.pcs = None
    out = sw.prepare().solve(restart=cf.RESTART, tol=cf.TOL_REF, maxit=cf.MAXIT_REF, prec="fp64")
    # the stop is on the preconditioned residual; the true one ends at its FP64 floor (a few 1e-12),
    # as the oracle's does
    assert np.all(out["relres"] < 1e-11), out["relres"]
    x64 = out["x"]
    # the points' sensitivity to the spectrum's rounding noise (see the module docstring)
    sw.precon_kind = "schur_invert_df"
    sw.pcs = None
    ri = sw.prepare().solve(restart=cf.RESTART, tol=cf.TOL_SENS, maxit=cf.MAXIT_REF, prec="fp32")
    assert np.all(ri["flag"] == 0), ri["relres"]
    for key in ("R", "L"):
        err = rel_port(out[key], fx[key])
        bound = np.maximum(cf.bound(fx, key, FP64_TOL), 2 * rel_port(out[key], ri[key]))
        assert np.all(err < bound), (key, err, bound, fx["sens_" + key])
        # no point may be left undetermined at the mixed path's accuracy bar (the spiral's 20 GHz R,
        # the most sensitive, moves by 6e-8 with the spectrum's rounding noise)
        assert np.all(bound < MIXED_TOL), (key, bound)
    dx = float(np.linalg.norm(x64 - ri["x"]) / np.linalg.norm(x64))
    check_x(out, fx, int(fx["nc"]), max(FP64_TOL, 10 * float(fx["sens_x"]), 2 * dx))


@pytest.mark.parametrize("name", NAMES)
def test_mixed_matches_oracle(lib, name):
    fx, sw = sweep_of(lib, name)
    sw.precon_kind = "schur_invert_df"
    sw.pcs = None
    out = sw.prepare().solve(restart=50, tol=1e-10, maxit=10, prec="fp32")
    assert np.all(out["flag"] == 0), out["relres"]
    assert np.all(rel_port(out["R"], fx["R"]) < cf.bound(fx, "R", MIXED_TOL))
    assert np.all(rel_port(out["L"], fx["L"]) < cf.bound(fx, "L", MIXED_TOL))
    check_x(out, fx, int(fx["nc"]), MIXED_TOL)


def test_bar_own_settings_match_oracle(lib):
    """C1 at tol 1e-8, restart 50, maxit 10: the oracle's iteration counts and its x, R, L."""
    name = "bar_64x16x16"
    fx, sw = sweep_of(lib, name)
    sw.precon_kind = "schur_invert"
    sw.pcs = None
    out = sw.prepare().solve(restart=50, tol=float(fx["cfg_tol"]), maxit=10, prec="fp64")
    inner = out["iter"][:, 0] + (out["iter"][:, 1] - 1) * 50
    np.testing.assert_array_equal(inner, fx["cfg_iters"].ravel())
    assert np.all(rel_port(out["R"], fx["cfg_R"]) < FP64_TOL)
    assert np.all(rel_port(out["L"], fx["cfg_L"]) < FP64_TOL)
    check_x(out, fx, int(fx["nc"]), OWN_SETTINGS_X_TOL, prefix="cfgx_")


def test_release_sweeps():
    """Frees the last configuration's device state before the tests that follow."""
    for k in list(_SWEEPS):
        _SWEEPS.pop(k)[1].geom.close()
