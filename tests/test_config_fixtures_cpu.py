"""The oracle fixtures of the benchmark configurations: known answers, consistency, reproducibility."""
import numpy as np
import pytest

import config_fixtures as cf


def fixture_or_skip(name):
    import os

    if not os.path.exists(cf.path(name)):
        pytest.skip(f"fixture {cf.path(name)} not generated")
    return cf.load(name)


@pytest.mark.parametrize("name", list(cf.CONFIGS))
def test_fixture_is_consistent(name):
    fx = fixture_or_skip(name)
    from voxhenry_gb300 import geometry

    w = geometry.WORKLOADS[name]()
    np.testing.assert_array_equal(fx["freqs"], w.freqs[fx["freq_idx"]])
    P = int(fx["ports"])
    assert fx["Y"].shape == (len(fx["freqs"]), P, P)
    Z = np.linalg.inv(fx["Y"])
    np.testing.assert_allclose(fx["R"], np.abs(Z.real), rtol=1e-12)
    np.testing.assert_allclose(fx["L"], np.abs(Z.imag) / (2 * np.pi * fx["freqs"])[:, None, None], rtol=1e-12)
    # pgmres stops on the preconditioned residual (pgmres.m:121-149); the true relative residual it
    # reports afterwards (pgmres.m:181) can sit a few times above tol, and at tol 1e-14 it stops at the
    # FP64 floor of the point (3e-12 to 7e-12 on the spiral)
    assert np.all(fx["relres"] <= max(100 * float(fx["tol"]), 1e-11))
    assert fx["x_curr_sketch"].shape == (len(fx["freqs"]) * P, cf.SKETCH_K)
    # the conditioning measure: every point is determined far below the mixed path's 1e-6 bar
    assert fx["sens_R"].shape == (len(fx["freqs"]),) and float(fx["sens_x"]) < 1e-7
    assert fx["sens_R"].max() < 1e-7 and fx["sens_L"].max() < 1e-7


def test_bar_dc_resistance_known_answer():
    """C1 at 1 kHz (skin depth ~2 mm >> 8 um): R = l / (sigma A) of the 32 x 8 x 8 um bar."""
    fx = fixture_or_skip("bar_64x16x16")
    assert fx["freqs"][0] == pytest.approx(1e3)
    r_dc = 64 * 0.5e-6 / (5.8e7 * (16 * 0.5e-6) * (16 * 0.5e-6))
    assert abs(fx["R"][0, 0, 0] - r_dc) / r_dc < 1e-6
    # resistance rises with frequency (skin and proximity effect), inductance falls
    assert fx["R"][-1, 0, 0] > fx["R"][0, 0, 0]
    assert fx["L"][-1, 0, 0] < fx["L"][0, 0, 0]


def test_two_bars_dc_resistance_known_answer():
    """C3 at 1 kHz: each 100 x 10 x 10 um bar's self resistance is l / (sigma A)."""
    fx = fixture_or_skip("two_bars_128x64x32")
    assert fx["freqs"][0] == pytest.approx(1e3)
    for p, sigma in enumerate((5.8e7, 3.5e7)):
        r_dc = 100e-6 / (sigma * 10e-6 * 10e-6)
        assert abs(fx["R"][0, p, p] - r_dc) / r_dc < 1e-6


def test_bar_fixture_reproduces_with_the_oracle():
    """The committed oracle reproduces the C1 fixture at 1 kHz and 10 GHz (the first and last point)."""
    fx = fixture_or_skip("bar_64x16x16")
    from oracle import circulant, solver, structure
    from voxhenry_gb300 import geometry

    w = geometry.bar()
    S = structure.build_system(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght)
    fN, st2 = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    sel = [0, len(fx["freqs"]) - 1]
    out = solver.solve_frequencies(S, fN, st2, fx["freqs"][sel], restart=cf.RESTART, maxit=cf.MAXIT_REF,
                                   tol=cf.TOL_REF, keep_x=True)
    np.testing.assert_allclose(out["R"], fx["R"][sel], rtol=1e-11)
    np.testing.assert_allclose(out["L"], fx["L"][sel], rtol=1e-11)
    d = cf.compare(np.stack(out["x"]), int(fx["nc"]), {k: v[sel] if k.endswith(("sample", "blocks", "norm", "sketch"))
                                                      else v for k, v in fx.items()})
    # x to 1e-10: the fixtures' tensor spectrum came from one FFT implementation, the oracle's from the
    # multithreaded SciPy one, whose roundings differ at ~1e-12 after a 44-iteration solve
    assert d["curr_sketch"] < 1e-10 and d["phi_sketch"] < 1e-10, d


def test_sketch_estimates_the_relative_difference():
    """|G (x1 - x2)| / |G x2| tracks |x1 - x2| / |x2| within the stated ~25 % for 64 rows."""
    rng = np.random.default_rng(11)
    n, nc = 20000, 12000
    X = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
    fx = {"x_" + k: v for k, v in cf.fingerprint(X, nc).items()}
    for eps in (1e-6, 1e-9):
        E = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
        E *= eps * np.linalg.norm(X, axis=1, keepdims=True) / np.linalg.norm(E, axis=1, keepdims=True)
        d = cf.compare(X + E, nc, fx)
        true_c = np.max(np.linalg.norm(E[:, :nc], axis=1) / np.linalg.norm(X[:, :nc], axis=1))
        assert 0.7 * true_c < d["curr_sketch"] < 1.3 * true_c, (d, true_c)
    assert cf.compare(X, nc, fx)["curr_sketch"] == 0.0
