"""Pins the CPU oracle against the reference's own published outputs (CPU only)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_vhr_text
from oracle import circulant, solver, structure, vhr

REF = np.load(os.path.join(GOLDEN, "reference_results.npz"))
NUMEX1 = "straight_cond1_len30.0u_wid10.0u_dist20.0u.vhr"


@pytest.fixture(scope="module")
def numex1():
    inp = vhr.read_vhr_text(golden_vhr_text(NUMEX1))
    S = structure.build_system(inp.sigma_e, inp.lambdaL, inp.dx, inp.pnt_lft, inp.pnt_rght, inp.pnt_well_cond)
    fN, st = circulant.generate_circulant_tensor(inp.dx, 1.0, S.L, S.M, S.N)
    return inp, S, fN, st


def test_reader_numex1(numex1):
    inp, S, _, _ = numex1
    assert inp.sigma_e.shape == (60, 20, 20)
    assert inp.dx == 5e-7 and inp.num_ports == 1
    np.testing.assert_array_equal(inp.freq, REF["numex1_freq"])
    assert S.nv == 24000 and S.num_nodes == 74800 and S.nc == 120000
    assert S.Ar.shape == (74000, 120000)


def test_panel_numbering_matches_reference(numex1):
    """Ae_only_leaving / Ae_only_entering_bndry pin lse_generate_panelIDs + lse_compute_Ae_matrix."""
    from tests.golden.make_golden import csc_digest
    _, S, _, _ = numex1
    for nm in ("Ae_only_leaving", "Ae_only_entering_bndry"):
        A = getattr(S, nm)
        assert A.nnz == int(REF[f"numex1_{nm}_nnz"])
        assert tuple(A.shape) == tuple(REF[f"numex1_{nm}_shape"])
        assert csc_digest(A) == str(REF[f"numex1_{nm}_digest"])


def test_rl_and_current_match_reference(numex1):
    """R, L at 1 MHz and 2.5 GHz and the 2.5 GHz current solution vs data_*.mat."""
    _, S, fN, st = numex1
    fr = REF["numex1_freq"]
    sel = [24, 37]                       # 1 MHz, 2.5 GHz
    out = solver.solve_frequencies(S, fN, st, fr[sel], keep_x=True)
    for i, k in enumerate(sel):
        gold = REF["numex1_RjL"][k]
        assert abs(out["R"][i, 0, 0] / gold.real - 1) < 1e-8
        assert abs(out["L"][i, 0, 0] / gold.imag - 1) < 1e-8
    x = out["x"][1]
    idx = REF["numex1_x_sample_idx"]
    np.testing.assert_allclose(x[idx], REF["numex1_x_sample"], rtol=0, atol=1e-6 * np.abs(REF["numex1_x_sample"]).max())
    nc = S.nc
    norms = np.array([np.linalg.norm(x[k * nc // 5:(k + 1) * nc // 5]) for k in range(5)])
    np.testing.assert_allclose(norms, REF["numex1_x_block_norms"], rtol=1e-6)


def test_dc_resistance_and_fasthenry(numex1):
    """R(DC) = l / (sigma A) for the 30 x 10 x 10 um bar; L within 0.2 % of FastHenry."""
    _, S, fN, st = numex1
    out = solver.solve_frequencies(S, fN, st, np.array([1.0]))
    r_dc = 30e-6 / (5.8e7 * 10e-6 * 10e-6)
    assert abs(out["R"][0, 0, 0] / r_dc - 1) < 1e-9
    fh = REF["numex1_fasthenry"]
    l_fh = fh[0, 2]
    assert abs(out["L"][0, 0, 0] / l_fh - 1) < 2e-3


def test_reference_rl_table_is_consistent():
    """The published numex1 table: DC R equals l/(sigma A) to 6 digits; L falls with f."""
    rjl = REF["numex1_RjL"]
    assert abs(rjl[0].real / (30e-6 / (5.8e7 * 1e-10)) - 1) < 1e-6
    assert np.all(np.diff(rjl.imag[20:]) <= 1e-20)
