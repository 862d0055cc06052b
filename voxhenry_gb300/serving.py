"""Serving of extraction requests on one GPU (the serving configuration of the benchmark).

A seeded stream of requests -- straight bars, voxelised cylindrical wires and square spirals,
grids from 16^3 up to about 256x256x16, voxel 0.5-2 um, sigma 3.5e7-5.8e7 S/m, 1-4 ports and
1-64 log-spaced frequencies in [1 kHz, 20 GHz] -- is served one request at a time in arrival
order.  A request is the executer's whole job (VoxHenry_executer.m:151-329): setup (panel ids,
incidence, port rows, circulant tensor on the device), the Schur factors of its frequencies, the
batched mixed-precision solve and R, L.  Admission is by device-memory footprint: a request whose
factors and Krylov spaces would not fit the budget is split into frequency chunks.

Latency = queueing + service.  Service times are measured; arrivals are a seeded Poisson stream
at a given fraction of the measured capacity, and the single-server FIFO recursion (Lindley)
start_i = max(arrival_i, finish_(i-1)), finish_i = start_i + service_i gives each latency.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from . import _lib, executer, geometry, structure

SEED = 20261203


@dataclass
class Request:
    rid: int
    kind: str
    workload: geometry.Workload

    @property
    def freq_points(self) -> int:
        return len(self.workload.freqs)


def _parallel(kind: str, n: int, L: int, size: int, dx: float, sigma: float, freqs) -> geometry.Workload:
    """n parallel conductors along x (square bars of side `size`, or wires of diameter `size`),
    one port each from the x = 1 to the x = L faces."""
    pitch = size + 2
    M = max(16, n * pitch + 2)
    N = max(16, size + 4) if kind == "cylinder" else 16
    s = np.zeros((L, M, N), order="F")
    ports_l, ports_r = [], []
    for p in range(n):
        y0 = 2 + p * pitch
        if kind == "bar":
            z0 = (N - size) // 2
            s[:, y0:y0 + size, z0:z0 + size] = sigma
            occ = np.zeros(s.shape, bool)
            occ[:, y0:y0 + size, z0:z0 + size] = True
        else:
            cy, cz = y0 + (size - 1) / 2.0, (N - 1) / 2.0
            j = np.arange(M)[:, None]
            k = np.arange(N)[None, :]
            disc = (j - cy) ** 2 + (k - cz) ** 2 <= (size / 2.0) ** 2
            s[:, disc] = sigma
            occ = np.zeros(s.shape, bool)
            occ[:, disc] = True
        m1 = np.zeros(s.shape, bool)
        m1[0] = occ[0]
        m2 = np.zeros(s.shape, bool)
        m2[-1] = occ[-1]
        ports_l.append(geometry.face_nodes(m1, "-x"))
        ports_r.append(geometry.face_nodes(m2, "+x"))
    return geometry.Workload(kind, s, dx, ports_l, ports_r, np.asarray(freqs, float))


def request_stream(n: int, seed: int = SEED) -> list[Request]:
    """n seeded requests of the serving configuration."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        kind = ("bar", "cylinder", "spiral")[int(rng.integers(3))]
        dx = float(rng.uniform(0.5e-6, 2e-6))
        sigma = float(rng.uniform(3.5e7, 5.8e7))
        nfreq = int(rng.integers(1, 65))
        freqs = np.logspace(3, np.log10(2e10), nfreq)
        if kind == "spiral":
            turns = int(rng.integers(2, 7))
            width = int(rng.integers(2, 6))
            pitch = width + 2
            side = int(min(256, max(16, 2 * 2 + 2 * turns * pitch + 2 * width + 4 + int(rng.integers(0, 24)))))
            w = geometry.square_spiral(L=side, M=side, N=8, dx=dx, turns=turns, width=width, thick=4, space=2,
                                       inset=2, sigma=sigma, freqs=freqs)
        else:
            nport = int(rng.integers(1, 5))
            L = int(rng.integers(16, 257))
            size = int(rng.integers(4, 41)) if kind == "cylinder" else int(rng.integers(2, 13))
            w = _parallel(kind, nport, L, size, dx, sigma, freqs)
        out.append(Request(i, kind, w))
    return out


def fifo_latencies(service: np.ndarray, arrivals: np.ndarray) -> np.ndarray:
    """Latency of each request through one server in arrival order (Lindley's recursion)."""
    lat = np.empty(len(service))
    free = -np.inf
    for i, (a, s) in enumerate(zip(arrivals, service)):
        start = max(a, free)
        free = start + s
        lat[i] = free - a
    return lat


def poisson_arrivals(n: int, rate: float, seed: int = SEED) -> np.ndarray:
    """n arrival times of a Poisson stream of `rate` requests per second, starting at 0."""
    rng = np.random.default_rng(seed + 1)
    gaps = rng.exponential(1.0 / rate, size=n)
    return np.concatenate([[0.0], np.cumsum(gaps[:-1])])


def footprint_bytes(prob, nfreq: int, restart: int = 50, exact: bool = True) -> int:
    """Device bytes of one request: tensor spectra (complex128, complex64 and the double-float copy),
    the Schur factors, the Krylov bases and the solver's work vectors.  exact: factor bytes from the
    symbolic analysis (vh_schur_analyze); else an upper bound of 64 stored entries per panel unknown
    (the nested-dissection fronts of these grids store under 50)."""
    P = 8 * prob.L * prob.M * prob.N
    n = prob.Ar.shape[0] + prob.Ar.shape[1]
    B = nfreq * prob.num_ports
    # Krylov basis (restart + 1 vectors), GMRES and refinement work vectors (~20), FFT scratch of
    # the complex128 product (two 5-component half-padded spectra per RHS)
    base = 7 * P * (16 + 8 + 16) + B * n * 16 * (restart + 24) + B * 5 * P * 16 // 2
    if not exact:
        return int(base + nfreq * 64 * prob.Ar.shape[0] * 8)
    lib = _lib.load()
    A = prob.Ar.tocsc()
    A.sort_indices()
    jc = np.ascontiguousarray(A.indptr, dtype=np.int64)
    ir = np.ascontiguousarray(A.indices, dtype=np.int64)
    pr = np.ascontiguousarray(A.data, dtype=np.float64)
    idx = np.ascontiguousarray(prob.idxS, dtype=np.int64)
    fb = C.c_int64()
    _lib.check(lib.vh_schur_analyze(prob.L, prob.M, prob.N, idx.size, _lib.i64ptr(idx), A.shape[0], _lib.i64ptr(jc),
                                    _lib.i64ptr(ir), _lib.dptr(pr), None, None, None, None, C.byref(fb)))
    return int(base + nfreq * fb.value)


def serve(requests, budget_bytes: int, prec: str = "fp32", tol: float = 1e-9, restart: int = 50,
          max_seconds: float | None = None, min_requests: int = 1) -> dict:
    """Serves the requests back to back (stopping once the service time passes max_seconds, after at
    least min_requests); returns their service times (s), frequency points and convergence."""
    import torch

    service, points, ok = [], [], []
    for req in requests:
        if max_seconds is not None and len(service) >= min_requests and sum(service) >= max_seconds:
            break
        w = req.workload
        t0 = time.perf_counter()
        prob = structure.problem_from_workload(w)
        nf = len(w.freqs)
        # admission: the frequencies that fit the budget together (the exact factor size only when
        # the cheap bound does not fit)
        need = footprint_bytes(prob, nf, restart, exact=False)
        if need > budget_bytes // 2:
            need = footprint_bytes(prob, nf, restart, exact=True)
        chunk = nf if need <= budget_bytes else max(1, int(budget_bytes // max(1, need // nf)))
        flags = []
        c0 = 0
        while c0 < nf:
            sw = None
            try:
                sw = executer.Sweep(prob, w.freqs[c0:c0 + chunk], want_fp32=True,
                                    precon="schur_invert_df" if prec == "fp32" else "schur_invert")
                out = sw.prepare().solve(restart=restart, tol=tol, maxit=10, prec=prec)
            except _lib.VHError as e:   # the model missed: halve the chunk and retry (OOM is a status)
                if e.status != _lib.VH_ERR_OOM or chunk == 1:
                    raise
                chunk = max(1, chunk // 2)
                continue
            finally:
                if sw is not None:
                    for p in sw.pcs or []:
                        p.close()
                    sw.geom.close()
            flags.append(np.asarray(out["flag"]))
            c0 += chunk
        torch.cuda.synchronize()
        service.append(time.perf_counter() - t0)
        points.append(nf)
        ok.append(bool(np.all(np.concatenate(flags) == 0)))
    return {"service_s": np.array(service), "freq_points": np.array(points), "converged": np.array(ok)}


def summarize(served: dict, load: float = 0.8, seed: int = SEED) -> dict:
    """p50 / p99 latency and throughput of the served requests under Poisson arrivals at `load` times
    the measured capacity."""
    s = served["service_s"]
    rate = load / float(np.mean(s))
    arr = poisson_arrivals(len(s), rate, seed)
    lat = fifo_latencies(s, arr)
    makespan = float(arr[-1] + lat[-1])
    return {"requests": int(len(s)), "offered_load": load, "arrival_rate_per_s": round(rate, 4),
            "p50_latency_s": round(float(np.percentile(lat, 50)), 4),
            "p99_latency_s": round(float(np.percentile(lat, 99)), 4),
            "freq_points_per_s": round(float(served["freq_points"].sum()) / makespan, 3),
            "service_p50_s": round(float(np.percentile(s, 50)), 4),
            "all_converged": bool(np.all(served["converged"]))}
