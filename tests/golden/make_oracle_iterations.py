"""Write the oracle's GMRES iteration counts at every frequency of a benchmark configuration
(tests/golden/oracle_iterations.npz, one int array per workload name).

    python tests/golden/make_oracle_iterations.py [workload ...]   (default: ring_512x512x16)

The oracle (oracle/solver.py: pgmres with the schur_invert preconditioner, the restatement of
pgmres.m and VoxHenry_executer.m:215-329) solves each frequency of the workload at the benchmark's
GMRES settings (tol 1e-10, restart 50, maxit 10) and the total inner iterations per frequency (the
largest over its ports) are stored, with the R and L it reached.  The CPU reference arm of bench.py
times a bounded sample per frequency (the factorisation and two iterations) and scales it to a whole
frequency point with these counts.  Existing entries of other workloads are kept.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import circulant, solver, structure  # noqa: E402
from voxhenry_gb300 import geometry  # noqa: E402

OUT = os.path.join(HERE, "oracle_iterations.npz")
TOL, RESTART, MAXIT = 1e-10, 50, 10


def main(names):
    data = {}
    if os.path.exists(OUT):
        with np.load(OUT) as z:
            data = {k: z[k] for k in z.files}
    for name in names or ["ring_512x512x16"]:
        w = geometry.WORKLOADS[name]()
        S = structure.build_system(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght)
        fN, st2 = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
        P = S.rhs.shape[1]
        its, R, L, secs = [], [], [], []
        for f in w.freqs:
            t0 = time.perf_counter()
            out = solver.solve_frequencies(S, fN, st2, np.array([f]), restart=RESTART, maxit=MAXIT, tol=TOL)
            secs.append(time.perf_counter() - t0)
            its.append(max(i[2] for i in out["iters"]))
            R.append(out["R"][0])
            L.append(out["L"][0])
            print(f"{name}: {f:.4g} Hz: {its[-1]} iterations, {secs[-1]:.1f} s", flush=True)
        data[name] = np.asarray(its, dtype=np.int64)
        data[name + "_R"] = np.asarray(R).reshape(len(w.freqs), P, P)
        data[name + "_L"] = np.asarray(L).reshape(len(w.freqs), P, P)
        data[name + "_seconds"] = np.asarray(secs)
        np.savez_compressed(OUT, **data)
        print("wrote", OUT, flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
