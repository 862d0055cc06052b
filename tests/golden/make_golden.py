"""Extract compact golden fixtures from the reference's published result files.

    python tests/golden/make_golden.py <reference tree>      (or VOXHENRY_REFERENCE=<tree>)

Run where the reference tree is present; the fixtures it writes are committed
next to it so that tests can run where the reference is absent.

Sources (paths within the reference project):
  results_numex1_straight_conductor/data_R_jL_mat.mat   R + jL at 41 frequencies
  results_numex1_straight_conductor/data_curr_plot.mat  solution x at 2.5 GHz (port 1) and
                                                         Ae_only_leaving / Ae_only_entering_bndry
  results_numex2_wire/data_R_jL_mat.mat                 R + jL (wire)
  results_numex1_straight_conductor/fasthenry_results_straight_conductor.m  FastHenry R + jL table
  Input_files/straight_cond1_len30.0u_wid10.0u_dist20.0u.vhr, wire_len2.0u_dia4.0u.vhr,
  wire_len50.0u_dia10.0u.vhr   (copied verbatim, gzip-compressed, as inputs)
"""
from __future__ import annotations

import gzip
import hashlib
import os
import re
import shutil
import sys

import numpy as np
import scipy.io as sio

HERE = os.path.dirname(os.path.abspath(__file__))


def csc_digest(A) -> str:
    A = A.tocsc()
    A.sort_indices()
    h = hashlib.sha256()
    h.update(np.asarray(A.shape, dtype=np.int64).tobytes())
    h.update(A.indptr.astype(np.int64).tobytes())
    h.update(A.indices.astype(np.int64).tobytes())
    h.update(A.data.astype(np.float64).tobytes())
    return h.hexdigest()


def main(ref: str) -> None:
    out = {}
    g = sio.loadmat(os.path.join(ref, "results_numex1_straight_conductor/data_R_jL_mat.mat"))
    out["numex1_freq"] = g["freq_all"].ravel().astype(np.float64)
    out["numex1_RjL"] = g["R_jL_mat"].ravel().astype(np.complex128)
    g2 = sio.loadmat(os.path.join(ref, "results_numex2_wire/data_R_jL_mat.mat"))
    out["numex2_freq"] = g2["freq_all"].ravel().astype(np.float64)
    out["numex2_RjL"] = g2["R_jL_mat"].ravel().astype(np.complex128)
    d = sio.loadmat(os.path.join(ref, "results_numex1_straight_conductor/data_curr_plot.mat"))
    x = d["x"].ravel().astype(np.complex128)
    nc = 120000
    out["numex1_x_len"] = np.int64(x.size)
    # every 97th current coefficient and the 2-norm of each of the 5 current blocks
    out["numex1_x_sample_idx"] = np.arange(0, nc, 97, dtype=np.int64)
    out["numex1_x_sample"] = x[out["numex1_x_sample_idx"]]
    out["numex1_x_block_norms"] = np.array([np.linalg.norm(x[k * nc // 5:(k + 1) * nc // 5]) for k in range(5)])
    for nm in ("Ae_only_leaving", "Ae_only_entering_bndry"):
        A = d[nm].tocsc()
        out[f"numex1_{nm}_digest"] = np.array(csc_digest(A))
        out[f"numex1_{nm}_nnz"] = np.int64(A.nnz)
        out[f"numex1_{nm}_shape"] = np.asarray(A.shape, dtype=np.int64)
    # FastHenry reference table: rows "f  R+Lj"
    txt = open(os.path.join(ref, "results_numex1_straight_conductor/fasthenry_results_straight_conductor.m")).read()
    rows = re.findall(r"^\s*([0-9.eE+-]+)\s+([0-9.eE+-]+)\+([0-9.eE+-]+)j", txt, flags=re.M)
    fh = np.array([[float(a), float(b), float(c)] for a, b, c in rows])
    out["numex1_fasthenry"] = fh
    np.savez_compressed(os.path.join(HERE, "reference_results.npz"), **out)
    for f in ("straight_cond1_len30.0u_wid10.0u_dist20.0u.vhr", "wire_len2.0u_dia4.0u.vhr",
              "wire_len50.0u_dia10.0u.vhr"):
        with open(os.path.join(ref, "Input_files", f), "rb") as src, gzip.open(os.path.join(HERE, f + ".gz"), "wb") as dst:
            shutil.copyfileobj(src, dst)
    print("wrote", sorted(out))


if __name__ == "__main__":
    tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VOXHENRY_REFERENCE")
    if not tree:
        sys.exit("usage: make_golden.py <reference tree> (or set VOXHENRY_REFERENCE)")
    main(tree)
