"""The product's .vhr reader and writer (voxhenry_gb300.vhr) vs the oracle's reader on the
reference's own input files, and write -> read round trips."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_vhr_text
from oracle import vhr as ovhr
from voxhenry_gb300 import vhr

FILES = ["straight_cond1_len30.0u_wid10.0u_dist20.0u.vhr", "wire_len2.0u_dia4.0u.vhr", "wire_len50.0u_dia10.0u.vhr"]


def same_model(m, o):
    np.testing.assert_array_equal(m.sigma_e, o.sigma_e)
    assert (m.lambdaL is None) == (o.lambdaL is None)
    if m.lambdaL is not None:
        np.testing.assert_array_equal(m.lambdaL, o.lambdaL)
    np.testing.assert_array_equal(m.freq, o.freq)
    assert m.dx == o.dx and m.num_ports == o.num_ports
    for a, b in zip(m.pnt_lft + m.pnt_rght, o.pnt_lft + o.pnt_rght):
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


@pytest.mark.parametrize("name", FILES)
def test_reader_matches_oracle_on_reference_inputs(name):
    text = golden_vhr_text(name)
    same_model(vhr.parse(text), ovhr.read_vhr_text(text))


@pytest.mark.parametrize("name", FILES)
def test_write_read_round_trip(name, tmp_path):
    m = vhr.parse(golden_vhr_text(name))
    p = str(tmp_path / "out.vhr.gz")
    vhr.write(p, m, title=name)
    same_model(vhr.read(p), m)
    same_model(ovhr.read_vhr_text(vhr.format_text(m)), m)   # the oracle reads what the writer writes


def test_superconductor_round_trip():
    rng = np.random.default_rng(1)
    sig = np.zeros((6, 5, 4), order="F")
    sig[1:5, 1:4, 1:3] = 5.8e7
    lam = np.where(sig > 0, 1e-7 * rng.uniform(1, 2, sig.shape), 0.0)
    m = vhr.VhrModel(sig, np.asfortranarray(lam), np.array([1e3, 1e6, 2.5e9]), 1e-6,
                     [np.array([[2, 2, 2, 1]])], [np.array([[5, 2, 2, 2]])], None, ["p1"])
    r = vhr.parse(vhr.format_text(m))
    np.testing.assert_allclose(r.lambdaL, m.lambdaL, rtol=1e-5)   # %g keeps 6 digits, as the reference writer
    np.testing.assert_array_equal(r.sigma_e, m.sigma_e)
    assert r.portnames == ["p1"]


def test_workload_from_vhr_builds_the_reference_system(tmp_path):
    """A .vhr file -> Workload -> native set-up gives the system the oracle builds from the same file."""
    from oracle import structure as ostruct
    from voxhenry_gb300 import geometry, structure

    text = golden_vhr_text(FILES[0])
    p = str(tmp_path / "in.vhr")
    with open(p, "w") as f:
        f.write(text)
    w = geometry.from_vhr(p)
    prob = structure.problem_from_workload(w)
    inp = ovhr.read_vhr_text(text)
    S = ostruct.build_system(inp.sigma_e, inp.lambdaL, inp.dx, inp.pnt_lft, inp.pnt_rght)
    np.testing.assert_array_equal(prob.idxS, S.idxS)
    assert (prob.Ar != S.Ar).nnz == 0
    np.testing.assert_array_equal(prob.rhs, S.rhs)
