"""Host-side nested dissection / multifrontal analysis of S = Ae A_inv Ae^T (CPU only)."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden_vhr_text
from oracle import structure, vhr


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import _lib

    return _lib


def analyze(_lib, L, M, N, idxS, Ar):
    lib = _lib.load()
    A = sp.csc_matrix(Ar)
    A.sort_indices()
    jc = np.ascontiguousarray(A.indptr, dtype=np.int64)
    ir = np.ascontiguousarray(A.indices, dtype=np.int64)
    pr = np.ascontiguousarray(A.data, dtype=np.float64)
    idx = np.ascontiguousarray(idxS, dtype=np.int64)
    nnz, fl, nf, mf, fb = C.c_int64(), C.c_double(), C.c_int(), C.c_int(), C.c_int64()
    st = lib.vh_schur_analyze(L, M, N, idx.size, _lib.i64ptr(idx), A.shape[0], _lib.i64ptr(jc), _lib.i64ptr(ir),
                              _lib.dptr(pr), C.byref(nnz), C.byref(fl), C.byref(nf), C.byref(mf), C.byref(fb))
    return st, dict(nnz=nnz.value, flops=fl.value, fronts=nf.value, max_front=mf.value, bytes=fb.value)


def test_numex1_analysis(lib):
    inp = vhr.read_vhr_text(golden_vhr_text("straight_cond1_len30.0u_wid10.0u_dist20.0u.vhr"))
    S = structure.build_system(inp.sigma_e, None, inp.dx, inp.pnt_lft, inp.pnt_rght)
    st, r = analyze(lib, S.L, S.M, S.N, S.idxS, S.Ar)
    assert st == 0
    # fill of the geometric nested dissection: below SuperLU's minimum-degree factor (12.3M)
    assert 1e6 < r["nnz"] < 1.2e7
    assert r["max_front"] <= 1200 and r["fronts"] > 100


def test_spiral_fronts_stay_small(lib):
    from voxhenry_gb300 import geometry

    w = geometry.square_spiral()
    S = structure.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    st, r = analyze(lib, S.L, S.M, S.N, S.idxS, S.Ar)
    assert st == 0 and r["max_front"] <= 400 and r["flops"] < 2e9


def test_rejects_foreign_matrix(lib):
    A = sp.random(30, 5 * 8, density=0.2, random_state=1, format="csc")
    A.data[:] = 0.25
    st, _ = analyze(lib, 2, 2, 2, np.arange(1, 9), A)
    assert st == 3   # VH_ERR_UNSUPPORTED
