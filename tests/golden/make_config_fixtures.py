"""Write the oracle fixtures of the benchmark configurations (tests/golden/config_<name>.npz).

    python tests/golden/make_config_fixtures.py [name ...]     (default: all four)

For each configuration of tests/golden/config_fixtures.CONFIGS it builds the seeded synthetic
workload (voxhenry_gb300.geometry: inputs only), then the oracle's own system (panel ids, Ae, port
rows, RHS: oracle/structure.py) and circulant tensor (oracle/circulant.py), and solves the selected
frequencies with the oracle's left-preconditioned pgmres (oracle/solver.py, the restatement of
pgmres.m / VoxHenry_executer.m:215-329) to tol 1e-12.  The oracle runs on the host cores only; the
ring (FFT grid 1024 x 1024 x 32) takes several minutes per frequency point.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import config_fixtures as cf  # noqa: E402

from oracle import circulant, solver, structure  # noqa: E402
from voxhenry_gb300 import geometry  # noqa: E402


def solve(S, fN, st2, freqs, tol, maxit):
    t0 = time.perf_counter()
    out = solver.solve_frequencies(S, fN, st2, freqs, restart=cf.RESTART, maxit=maxit, tol=tol, keep_x=True)
    t = time.perf_counter() - t0
    P = S.rhs.shape[1]
    X = np.stack(out["x"])                           # (F * P, n), frequency-major
    it = np.array([[i[2] for i in out["iters"][k * P:(k + 1) * P]] for k in range(len(freqs))], dtype=np.int64)
    rr = np.array([[i[3] for i in out["iters"][k * P:(k + 1) * P]] for k in range(len(freqs))])
    return out, X, it, rr, t


def make(name: str) -> None:
    spec = cf.CONFIGS[name]
    w = geometry.WORKLOADS[name]()
    t0 = time.perf_counter()
    S = structure.build_system(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght)
    fN, st2 = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    t_setup = time.perf_counter() - t0
    fi = np.asarray(spec["freq_idx"], dtype=np.int64)
    freqs = w.freqs[fi]
    res = {"name": np.array(name), "freq_idx": fi, "freqs": freqs, "grid": np.array([S.L, S.M, S.N]),
           "nv": np.int64(S.nv), "nc": np.int64(S.nc), "n": np.int64(S.n), "ports": np.int64(S.rhs.shape[1]),
           "tol": np.float64(cf.TOL_REF), "restart": np.int64(cf.RESTART), "maxit": np.int64(cf.MAXIT_REF),
           "t_setup": np.float64(t_setup)}
    out, X, it, rr, t = solve(S, fN, st2, freqs, cf.TOL_REF, cf.MAXIT_REF)
    res.update(Y=out["Y"], Z=out["Z"], R=out["R"], L=out["L"], iters=it, relres=rr, t_solve=np.float64(t))
    fp = cf.fingerprint(X, S.nc)
    res.update({"x_" + k: v for k, v in fp.items()})
    print(f"{name}: n={S.n} setup {t_setup:.1f} s, {len(freqs)} freqs x {S.rhs.shape[1]} ports to tol "
          f"{cf.TOL_REF:g} in {t:.1f} s, iterations {it.ravel().tolist()}", flush=True)
    # sensitivity: the same points solved to tol 1e-12
    o2, X2, it2, rr2, t2 = solve(S, fN, st2, freqs, cf.TOL_SENS, cf.MAXIT_REF)
    P = S.rhs.shape[1]
    rel_port = lambda a, b: np.array([np.abs(a[k] - b[k]).max() / np.abs(b[k]).max() for k in range(b.shape[0])])
    res["sens_R"] = rel_port(o2["R"], out["R"])
    res["sens_L"] = rel_port(o2["L"], out["L"])
    d = cf.compare(X2, S.nc, {"x_" + k: v for k, v in fp.items()})
    res["sens_x"] = np.float64(max(d["curr_sketch"], d["phi_sketch"]))
    print(f"{name}: sensitivity (tol {cf.TOL_SENS:g} vs {cf.TOL_REF:g}) R {res['sens_R'].tolist()} "
          f"L {res['sens_L'].tolist()} x {float(res['sens_x']):.2e} ({t2:.1f} s)", flush=True)
    if "config_tol" in spec:   # the configuration's own GMRES settings (restart 50, maxit 10)
        tc = spec["config_tol"]
        out, X, it, rr, t = solve(S, fN, st2, freqs, tc, 10)
        res.update(cfg_tol=np.float64(tc), cfg_R=out["R"], cfg_L=out["L"], cfg_iters=it, cfg_relres=rr)
        res.update({"cfgx_" + k: v for k, v in cf.fingerprint(X, S.nc).items()})
        print(f"{name}: at tol {tc:g}: {t:.1f} s, iterations {it.ravel().tolist()}", flush=True)
    np.savez_compressed(cf.path(name), **res)
    print("wrote", cf.path(name), os.path.getsize(cf.path(name)), "bytes", flush=True)


def main(names):
    for nm in names or list(cf.CONFIGS):
        make(nm)


if __name__ == "__main__":
    main(sys.argv[1:])
