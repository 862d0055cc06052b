"""Serving of extraction requests on one GPU with continuous batching (the serving configuration of
the benchmark).

A seeded stream of requests -- straight bars, voxelised cylindrical wires and square spirals,
grids from 16^3 up to about 256x256x16, voxel 0.5-2 um, sigma 3.5e7-5.8e7 S/m, 1-4 ports and
1-64 log-spaced frequencies in [1 kHz, 20 GHz] -- arrives over time.  A request is the executer's
whole job (VoxHenry_executer.m:151-329): setup (panel ids, incidence, port rows, circulant tensor on
the device), the Schur factors of its frequencies, the batched mixed-precision solve and R, L.

Server runs K slots.  Each slot owns a library context (its own CUDA stream and device block cache)
and a host worker thread; requests that arrive while others run are admitted, first come first
served, as soon as a slot is free and their device-memory footprint fits the budget left by the
running requests, so the work of up to K requests overlaps on the device.  A slot keeps the last
geometry it solved resident (tensor spectrum, Ae, symbolic analysis): a later request for the same
geometry on that slot skips the setup.  A request whose footprint exceeds the whole budget is solved in
frequency chunks.  Latency = completion - arrival, measured on the wall clock with the arrivals
replayed in real time.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import queue
import threading
import time
from collections import deque
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


def footprint_estimate(w: geometry.Workload, nfreq: int, restart: int = 50) -> int:
    """A request's device bytes from its workload alone, before its setup runs (the admission
    estimate; the worker replaces it with footprint_bytes once the setup has run): n <= 11 nv unknowns
    (5 currents and at most 6 panel nodes per voxel), and per node of the Schur factor about 0.45 times
    the nodes of a cut across the structure's longest axis (the nested-dissection fronts grow with the
    cross-section), at least 32; the tensor terms are exact."""
    L, M, N = w.sigma_e.shape
    P = 8 * L * M * N
    nv = int(np.count_nonzero(np.abs(w.sigma_e) > 1e-12))
    n = 11 * nv
    B = nfreq * len(w.pnt_lft)
    per_node = max(32.0, 0.45 * nv / max(L, M, N))
    return int(7 * P * (16 + 8 + 16) + B * n * 16 * (restart + 24) + B * 5 * P * 16 // 2 +
               nfreq * per_node * 4 * nv * 8)


def tensor_bytes(w: geometry.Workload) -> int:
    """Device bytes of a resident geometry's tensor spectra (complex128, complex64 and the pairs) and of
    the Toeplitz table of the complex64 z-pass (two floats per component, row and (kx, ky) of the
    voxel box's height, for boxes up to 16 rows)."""
    L, M, N = w.sigma_e.shape
    nz_rows = np.flatnonzero(np.abs(np.asarray(w.sigma_e)).sum(axis=(0, 1)) > 0)
    nz = int(nz_rows.max() - nz_rows.min() + 1) if nz_rows.size else 0
    table = 2 * 7 * nz * (2 * L) * (2 * M) * 4 if nz <= 16 else 0
    return int(7 * 8 * L * M * N * (16 + 8 + 16) + table)


def geometry_key(w: geometry.Workload) -> str:
    """Identity of a request's geometry (grid, voxel size, conductivities, ports): two requests with
    the same key share the tensor, Ae and the symbolic analysis."""
    k = w.meta.get("_geometry_key")
    if k is not None:
        return k
    h = hashlib.sha256()
    h.update(np.asarray(w.sigma_e.shape, dtype=np.int64).tobytes())
    h.update(np.float64(w.dx).tobytes())
    h.update(np.ascontiguousarray(w.sigma_e, dtype=np.float64).tobytes())
    if w.lambdaL is not None:
        h.update(np.ascontiguousarray(w.lambdaL, dtype=np.float64).tobytes())
    for side in (w.pnt_lft, w.pnt_rght):
        for rows in side:
            h.update(np.ascontiguousarray(rows, dtype=np.int64).tobytes())
    w.meta["_geometry_key"] = h.hexdigest()
    return w.meta["_geometry_key"]


@dataclass
class Served:
    rid: int
    arrival: float           # s after the run's start
    start: float = 0.0
    finish: float = 0.0
    slot: int = -1
    freq_points: int = 0
    reused_geometry: bool = False
    chunks: int = 1
    R: np.ndarray | None = None
    L: np.ndarray | None = None
    flags: np.ndarray | None = None
    error: str | None = None

    @property
    def latency(self):
        return self.finish - self.arrival


class Slot:
    """A library context (CUDA stream) and the geometry it keeps resident."""

    def __init__(self, index: int):
        from . import vie

        self.index = index
        self.ctx = vie.Context(0)
        self.key = None
        self.sweep = None
        self.prob = None

    def drop(self):
        if self.sweep is not None:
            for p in self.sweep.pcs or []:
                p.close()
            self.sweep.geom.close()
        self.sweep, self.key, self.prob = None, None, None

    def close(self):
        self.drop()
        self.ctx.close()


def solve_request(slot: Slot, req: Request, rec: Served, budget: int, prec="fp32", tol=1e-9, restart=50,
                  reserve=None):
    """The executer's job for one request on one slot: setup (or the slot's resident geometry), the
    factors and the batched solve of its frequencies (in chunks when they do not fit `budget`), R and L.
    reserve(bytes): tells the scheduler the request's exact footprint once the setup has run."""
    w = req.workload
    key = geometry_key(w)
    nf = len(w.freqs)
    kind = "schur_invert_df" if prec == "fp32" else "schur_invert"
    if slot.key == key and slot.sweep is not None:
        rec.reused_geometry = True
    else:
        slot.drop()
        slot.prob = structure.problem_from_workload(w, ctx=slot.ctx)
    need = footprint_bytes(slot.prob, nf, restart)   # host-only symbolic analysis (vh_schur_analyze)
    if reserve is not None:
        reserve(need)
    chunk = nf if need <= budget else max(1, int(nf * budget // need))
    if slot.sweep is None:
        slot.sweep = executer.Sweep(slot.prob, w.freqs[:chunk], want_fp32=True, precon=kind, ctx=slot.ctx)
        slot.key = key
    sw = slot.sweep
    Rs, Ls, flags = [], [], []
    c0 = 0
    rec.chunks = 0
    while c0 < nf:
        sw.set_frequencies(w.freqs[c0:c0 + chunk])
        try:
            out = sw.prepare().solve(restart=restart, tol=tol, maxit=10, prec=prec)
        except _lib.VHError as e:   # the bound missed (or another slot holds the memory): smaller chunks
            for p in sw.pcs or []:
                p.close()
            sw.pcs = None
            slot.ctx.trim()
            if e.status != _lib.VH_ERR_OOM or chunk == 1:
                raise
            chunk = max(1, chunk // 2)
            continue
        for p in sw.pcs:
            p.close()
        sw.pcs = None
        Rs.append(out["R"])
        Ls.append(out["L"])
        flags.append(np.asarray(out["flag"]))
        c0 += chunk
        rec.chunks += 1
    rec.R, rec.L, rec.flags = np.concatenate(Rs), np.concatenate(Ls), np.concatenate(flags)
    rec.freq_points = nf


class Server:
    """Continuous-batching extraction server: `slots` requests in flight, admitted first come first
    served as slots and device memory free up.  `solve` is the per-request work (solve_request; a test
    may pass a host-only stand-in together with slot_factory)."""

    def __init__(self, slots: int = 3, budget_bytes: int | None = None, prec: str = "fp32", tol: float = 1e-9,
                 restart: int = 50, solve=None, slot_factory=None):
        if budget_bytes is None:
            import torch

            free, _ = torch.cuda.mem_get_info()
            budget_bytes = int(0.8 * free)
        self.budget = int(budget_bytes)
        self.prec, self.tol, self.restart = prec, tol, restart
        self.solve = solve or (lambda slot, req, rec, budget, reserve: solve_request(slot, req, rec, budget, prec,
                                                                                     tol, restart, reserve))
        self.slots = [(slot_factory or Slot)(i) for i in range(slots)]
        self.max_in_flight = 0

    def close(self):
        for s in self.slots:
            s.close()

    def _need(self, req):
        w = req.workload
        return min(self.budget, footprint_estimate(w, len(w.freqs), self.restart))

    def run(self, requests, arrivals=None, time_limit: float | None = None) -> list:
        """Serves `requests` arriving at `arrivals` (s after the start; None: all at once), replayed on
        the wall clock.  Returns one Served record per request, in request order (a request not yet
        admitted when time_limit passes is left out)."""
        n = len(requests)
        arrivals = np.zeros(n) if arrivals is None else np.asarray(arrivals, dtype=np.float64)
        recs = [Served(r.rid, float(a)) for r, a in zip(requests, arrivals)]
        done_q: queue.Queue = queue.Queue()
        pending: deque = deque()
        free_slots = list(self.slots)
        reserved = {}
        lock = threading.Lock()
        in_flight = 0
        nxt = 0
        finished = 0
        admitted = 0
        share = self.budget // max(1, len(self.slots))
        t0 = time.perf_counter()

        def reserve_for(slot):
            def reserve(nbytes):   # the exact footprint, once the request's setup has run
                with lock:
                    reserved[slot.index] = min(self.budget, int(nbytes))
            return reserve

        def worker(slot, i):
            rec = recs[i]
            try:
                self.solve(slot, requests[i], rec, self.budget, reserve_for(slot))
                # the slot's block cache keeps the request's solver buffers: hand them back when they
                # exceed the slot's share of the budget (the resident geometry stays)
                if hasattr(slot, "ctx") and slot.ctx.memory()[1] > share // 2:
                    slot.ctx.trim()
            except Exception as e:   # recorded; the request counts as failed
                rec.error = f"{type(e).__name__}: {e}"
            rec.finish = time.perf_counter() - t0
            done_q.put((slot, i))

        while finished < admitted or nxt < n or pending:
            now = time.perf_counter() - t0
            while nxt < n and arrivals[nxt] <= now:
                pending.append(nxt)
                nxt += 1
            if time_limit is not None and now > time_limit:
                pending.clear()
                nxt = n
            # admission: the oldest pending request, when a slot is free and its footprint fits what the
            # running requests leave (the head waits for memory rather than being overtaken)
            while pending and free_slots:
                i = pending[0]
                need = self._need(requests[i])
                key = geometry_key(requests[i].workload)
                slot = next((s for s in free_slots if s.key == key), None)
                if slot is None:   # prefer a slot holding no geometry, else the least recently used
                    slot = next((s for s in free_slots if s.key is None), free_slots[0])
                with lock:
                    others = sum(v for k, v in reserved.items() if k != slot.index)
                if need > self.budget - others:
                    # idle slots give up their resident geometries before the head waits for memory
                    for s in [s for s in free_slots if s is not slot and getattr(s, "key", None) is not None]:
                        s.drop()
                        with lock:
                            reserved[s.index] = 0
                    with lock:
                        others = sum(v for k, v in reserved.items() if k != slot.index)
                    if need > self.budget - others:
                        break
                pending.popleft()
                free_slots.remove(slot)
                with lock:
                    reserved[slot.index] = need
                recs[i].start = time.perf_counter() - t0
                recs[i].slot = slot.index
                in_flight += 1
                admitted += 1
                self.max_in_flight = max(self.max_in_flight, in_flight)
                threading.Thread(target=worker, args=(slot, i), daemon=True).start()
            wait = None
            if nxt < n:
                wait = max(0.0, arrivals[nxt] - (time.perf_counter() - t0))
            if finished < admitted:
                try:
                    slot, i = done_q.get(timeout=wait)
                except queue.Empty:
                    continue
                finished += 1
                in_flight -= 1
                # an idle slot's resident geometry still holds its tensor spectra
                with lock:
                    reserved[slot.index] = tensor_bytes(requests[i].workload) if getattr(slot, "key", None) else 0
                free_slots.append(slot)
            elif wait:
                time.sleep(wait)
        return [r for r in recs if r.finish > 0]


def summarize_run(recs, wall: float | None = None) -> dict:
    """p50 / p99 latency (completion - arrival, wall clock) and throughput of a run."""
    lat = np.array([r.latency for r in recs])
    pts = int(sum(r.freq_points for r in recs))
    span = wall if wall is not None else max(r.finish for r in recs) - min(r.arrival for r in recs)
    ok = all(r.error is None and r.flags is not None and np.all(r.flags == 0) for r in recs)
    return {"requests": len(recs), "freq_points": pts,
            "p50_latency_s": round(float(np.percentile(lat, 50)), 4),
            "p99_latency_s": round(float(np.percentile(lat, 99)), 4),
            "freq_points_per_s": round(pts / span, 3),
            "service_p50_s": round(float(np.percentile([r.finish - r.start for r in recs], 50)), 4),
            "reused_geometries": int(sum(r.reused_geometry for r in recs)),
            "all_converged": bool(ok),
            "errors": [r.error for r in recs if r.error][:3]}
