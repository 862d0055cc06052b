"""Benchmark: frequency points per second of the batched VIE sweep on one GB300.

Workload (the batched configuration of the reference's solve path): 4-turn square spiral coil on a
256 x 256 x 8 voxel grid (1 um voxels, 5 um trace, 4 voxels thick, 2 um turn spacing,
sigma = 5.8e7 S/m), one port across the spiral ends, 32 frequencies log-spaced 1 MHz - 20 GHz,
solved as 32 right-hand sides in one batch (GMRES tol 1e-9, restart 50).  A step is one sweep:
the Schur-complement factorisation of every frequency plus the batched Krylov solve and the
R, L extraction.  The circulant tensor, Ae and the symbolic analysis are set up once before the
timed region (resident in HBM).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value  = mixed precision (complex64 FFT matvec inside FP64 refinement), inputs on the device.
e2e    = the same through the host-buffer C ABI call (vh_gmres), copies included.
fp64   = the plain all-FP64 GPU path on the same workload (reported beside `value`).
--impl reference times the CPU restatement of the reference's algorithm (the oracle) on the host.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "freq-points/s, mixed-prec batched vs plain FP64 on GB300 @1e-6 R,L; p50/p99 lat"
UNIT = "freq-points/s"
# GMRES tolerance: the loosest that keeps R and L within 1e-6 of the converged solution for both the
# FP64 and the mixed path on this workload (tol 1e-8 leaves 3.8e-6 (FP64) / 5.1e-6 (mixed) in R, L;
# tol 1e-9 leaves 4.0e-7 / 7.6e-7, measured against a tol-1e-12 FP64 solve)
TOL = 1e-9
RESTART = 50
MAXIT = 10
# the mixed path's Schur factor and triangular solves run in double-float (FP32 pairs, ~48 bits) on
# GB300's FP32 pipes; its FP64 refinement residuals set the final accuracy
MIXED_PRECON = "schur_invert_df"
# factor sharing between neighbouring frequencies for the separately reported variant: A_inv (hence S)
# within 1e-4 of the group's factor; on this sweep it halves the factors at unchanged iteration counts
SHARE_TOL = 1e-4


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload():
    from voxhenry_gb300 import geometry

    w = geometry.square_spiral()
    cfg = {
        "workload": "square spiral coil, 4 turns, grid 256x256x8 (padded FFT grid 512x512x16), voxel 1 um, "
                    "trace 5 um x 4 voxels, spacing 2 um, sigma 5.8e7 S/m, 1 port, 32 freqs 1 MHz-20 GHz log",
        "grid": [256, 256, 8],
        "voxels": int((w.sigma_e > 0).sum()),
        "rhs_per_step": len(w.freqs),
        "gmres": {"tol": TOL, "restart": RESTART, "maxit": MAXIT, "preconditioner": "schur_invert (left)",
                  "schur_factor": {"mixed": "double-float (FP32 pairs)", "fp64": "fp64"}},
        "l2": "per-RHS vectors (~9.6 MB complex128 each) x 32 RHS and the 470 MB complex128 tensor exceed "
              "the 129 MB L2; no flush needed",
    }
    return w, cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def conv_traffic_from_profile(name, key="dram_bytes_per_rhs_matvec"):
    """DRAM bytes per RHS (matvec or preconditioner apply) from a committed ncu summary."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        with open(p) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return float(line.split(":")[1])
    except OSError:
        pass
    return None


def fft_algorithmic_bytes_per_rhs(nv, L, M, N, s, st, B):
    """Two-pass pruned separable model of one RHS-matvec: compact in/out, one forward and one inverse
    round trip of 5 spectra pruned to 2L x 2M x N, the 7-component tensor read once per batch of B."""
    lmn = L * M * N
    return s * (10 * nv) + s * (4 * 5 * 4 * lmn) + st * 7 * 8 * lmn / B


# ---------------------------------------------------------------------------------------------- ours
def run_ours(args, rank, world):
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import _lib, executer, structure, vie

    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", "0")))
    w, cfg = workload()
    if args.mixed_precon != MIXED_PRECON:
        cfg["gmres"]["schur_factor"]["mixed"] = "fp64"
    prob = structure.problem_from_workload(w)
    freqs = w.freqs
    sw = executer.Sweep(prob, freqs, want_fp32=True)
    g = sw.geom
    lib = g.ctx._lib
    stream = torch.cuda.ExternalStream(lib.vh_ctx_stream(g.ctx.handle))
    F = len(freqs)
    B = F * prob.num_ports
    n = g.n
    rhs = prob.rhs.astype(np.complex128)
    b_host = np.ascontiguousarray(np.stack([rhs[:, p] for f in range(F) for p in range(prob.num_ports)]))
    scale = np.ascontiguousarray(np.repeat(1j * 2 * np.pi * freqs * executer.MU0, prob.num_ports))
    zsl = np.ascontiguousarray(np.repeat(sw.zslot, prob.num_ports).astype(np.int32))
    tolv = np.full(B, TOL)
    b_dev = torch.from_numpy(b_host.view(np.float64)).cuda()
    x_dev = torch.empty_like(b_dev)
    rhs_dev = torch.from_numpy(prob.rhs.astype(np.float64)).cuda()
    ip = C.POINTER(C.c_int)
    flag = np.zeros(B, dtype=np.int32)
    relres = np.zeros(B)
    iters = np.zeros(2 * B, dtype=np.int32)
    nres = np.zeros(B, dtype=np.int32)

    st_all = (1j * 2 * np.pi * freqs * executer.MU0)[:, None] * np.asarray(prob.st2)[None, :]
    # entries of the Schur factor (for the preconditioner's algorithmic bytes); builds the symbolic
    # analysis before the timed region, as the warm-up would
    _pc = g.precons(st_all[:1], sw.zslot[:1], kind=args.mixed_precon)
    nnz_l = int(_pc[0].stats()["nnz_factor"])
    _pc[0].close()

    def precon_kind(prec):
        return args.mixed_precon if prec == "fp32" else "schur_invert"

    # factor sharing between neighbouring frequencies: reported as a separate line of the JSON unless
    # --share-tol asks for it in the headline mixed path
    def share_groups(tol):
        return executer.factor_share_groups([executer.a_inv_classes(prob, f) for f in freqs], tol)

    share_rep = np.arange(F)
    if args.share_tol is not None:
        share_rep = share_groups(args.share_tol)
        cfg["factor_sharing"] = {"share_tol": args.share_tol, "factors_per_step": int(len(np.unique(share_rep)))}

    def device_step(prec, tol=None, maxit=MAXIT, rep=None):
        """One sweep with device-resident inputs: factors + batched solve + R, L."""
        if rep is None:
            rep = share_rep if prec == "fp32" else np.arange(F)
        reps = np.unique(rep)
        made = g.precons(st_all[reps], sw.zslot[reps], kind=precon_kind(prec))
        by_rep = dict(zip(reps.tolist(), made))
        pcs = [by_rep[int(r)] for r in rep]
        parr = (C.c_void_p * B)(*[pcs[k // prob.num_ports].handle for k in range(B)])
        tv = tolv if tol is None else np.full(B, tol)
        st = lib.vh_gmres_device(g.handle, B, parr, C.c_void_p(b_dev.data_ptr()), _lib.cview(scale),
                                 zsl.ctypes.data_as(ip), RESTART, _lib.dptr(tv), maxit, 0, _lib.PREC[prec],
                                 C.c_void_p(x_dev.data_ptr()), flag.ctypes.data_as(ip), _lib.dptr(relres),
                                 iters.ctypes.data_as(ip), None, 0, nres.ctypes.data_as(ip))
        _lib.check(st, g.ctx.handle)
        with torch.cuda.stream(stream):
            xc = torch.view_as_complex(x_dev.view(B, n, 2))
            Y = torch.einsum("bn,np->bp", xc, rhs_dev.to(torch.complex128))   # Y(:, p) = sum rhs .* x
            Yh = Y.cpu().numpy().reshape(F, prob.num_ports, prob.num_ports).transpose(0, 2, 1)
        Z = np.linalg.inv(Yh)
        for p in made:
            p.close()
        return np.abs(Z.real), np.abs(Z.imag) / (2 * np.pi * freqs)[:, None, None], iters[0::2].copy()

    def timed(prec, steps, warm, profile=False, rep=None):
        for _ in range(warm):
            device_step(prec, rep=rep)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        if profile:
            _lib.check(lib.vh_ctx_profile(g.ctx.handle, 1), g.ctx.handle)
        l0 = lib.vh_launch_count()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push(f"timed_{prec}")
        e0.record(stream)
        t0 = time.perf_counter()
        out = None
        for _ in range(steps):
            out = device_step(prec, rep=rep)
        e1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        wall = time.perf_counter() - t0
        launches = lib.vh_launch_count() - l0
        prof = None
        if profile:
            ms = np.zeros(7)
            calls = np.zeros(7, dtype=np.int64)
            units = np.zeros(7, dtype=np.int64)
            _lib.check(lib.vh_ctx_profile_read(g.ctx.handle, _lib.dptr(ms), calls.ctypes.data_as(C.POINTER(C.c_int64)),
                                               units.ctypes.data_as(C.POINTER(C.c_int64)), 7), g.ctx.handle)
            _lib.check(lib.vh_ctx_profile(g.ctx.handle, 0), g.ctx.handle)
            prof = (ms, calls, units)
        ev_ms = e0.elapsed_time(e1)
        # the host waits for the device inside every step, so device time == wall time of the region
        t = max(ev_ms / 1e3, wall)
        if world > 1:
            tt = torch.tensor([t], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t = float(tt.item())
        return t, out, launches, prof

    if args.mixed_only:      # profiling aid: only the warm-up and timed mixed-precision steps
        timed("fp32", args.steps, args.warmup)
        return
    # accuracy reference: the FP64 GPU path converged to 1e-12 (untimed); the FP64 GPU path matches
    # the oracle to 1e-9 in the parity tests
    R_t, L_t, _ = device_step("fp64", tol=1e-12, maxit=40)
    clocks = ClockSampler(0)
    # warm-up + timed, mixed precision (headline) with live section timing
    clocks.start()
    t_mixed, out_mixed, launches, prof = timed("fp32", args.steps, args.warmup, profile=True)
    clk = clocks.stop()
    # plain FP64 GPU path on the same workload
    t_fp64, out_fp64, _, _ = timed("fp64", args.steps, args.warmup)
    # the mixed path with one factor per group of neighbouring frequencies (A_inv within 1e-4)
    shared = None
    if args.share_tol is None:
        rep_s = share_groups(SHARE_TOL)
        t_sh, out_sh, _, _ = timed("fp32", args.steps, args.warmup, rep=rep_s)
        shared = (rep_s, t_sh, out_sh)
    # e2e: the host-buffer C ABI call a user makes (Sweep -> vh_gmres), copies inside the region
    sw.pcs = None
    sw.precon_kind = precon_kind("fp32")
    for _ in range(args.warmup):
        sw.prepare(share_tol=args.share_tol).solve(restart=RESTART, tol=TOL, maxit=MAXIT, prec="fp32")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_out = None
    for _ in range(args.steps):
        sw.pcs = None
        # the previous result is released first, as a caller that keeps no earlier sweep does: its
        # page-locked x block then returns to the host cache and is reused instead of pinning anew
        e2e_out = None
        e2e_out = sw.prepare(share_tol=args.share_tol).solve(restart=RESTART, tol=TOL, maxit=MAXIT, prec="fp32")
    t_e2e = time.perf_counter() - t0

    R_m, L_m, it_m = out_mixed
    R_d, L_d, it_d = out_fp64

    def rl_err(R, L):
        return float(np.max(np.abs(R - R_t) / np.abs(R_t))), float(np.max(np.abs(L - L_t) / np.abs(L_t)))

    err_R, err_L = rl_err(R_m, L_m)
    err_R64, err_L64 = rl_err(R_d, L_d)
    err_e2e = max(rl_err(e2e_out["R"], e2e_out["L"]))
    pts = args.steps * F * world
    value = pts / t_mixed
    # roofline of the FFT matvec kernel groups (section times: CUDA events on the library stream)
    ms, calls, units = prof
    peak, peak_kind = measured_hbm_peak()
    sections = {name: {"ms": round(float(ms[i]), 3), "calls": int(calls[i]), "rhs": int(units[i])}
                for i, name in enumerate(["fft_conv_df", "fft_conv_c64", "incidence_spmv", "schur_factor",
                                          "precon_apply", "krylov_vectors", "tensor"])}
    step_ms_total = 1e3 * t_mixed
    dominant = max(sections, key=lambda k: sections[k]["ms"])

    def fft_roofline(sec, s, label, profile_name, note):
        conv_ms, conv_calls, conv_rhs = ms[sec], calls[sec], units[sec]
        if conv_calls == 0:
            return None
        avg_b = conv_rhs / conv_calls
        bytes_per_rhs = fft_algorithmic_bytes_per_rhs(prob.idxS.size, prob.L, prob.M, prob.N, s, s, avg_b)
        achieved = bytes_per_rhs * conv_rhs / (conv_ms / 1e3) / 1e9
        traffic = conv_traffic_from_profile(profile_name)
        return {"kernel": label, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "traffic": None if traffic is None else round(traffic * avg_b, 1),
                "traffic_source": f"profiles/{profile_name} (ncu, 4-RHS launch, scaled per RHS)",
                "algorithmic_bytes_per_launch": round(bytes_per_rhs * avg_b, 1),
                "avg_rhs_per_launch": round(avg_b, 2), "launches": int(conv_calls),
                "avg_launch_ms": round(conv_ms / conv_calls, 4),
                "share_of_step_time": round(conv_ms / step_ms_total, 4), "note": note}

    roof64 = fft_roofline(0, 16, "FFT circulant matvec in double-float (refinement residuals, VH_PREC_DF: all 5 "
                          "passes in pair arithmetic, pair storage between passes)", "fft_matvec_df_spiral.txt",
                          "pair-arithmetic passes issue-bound on the FP32 pipes, the z-pass half of the call; "
                          "frac is against HBM with the algorithmic bytes of the two-pass pruned model")
    roof32 = fft_roofline(1, 8, "FFT circulant matvec, complex64 (inner GMRES matvecs; 5 passes)",
                          "fft_matvec_c64_spiral.txt", "passes bound by shared-memory traffic and issue (Stockham "
                          "stages in shared memory; the register z-pass issue-bound)")
    # the preconditioner apply (double-float triangular solves and the SpMVs around them): per
    # RHS-apply the pair-precision factor is read once in each direction and the complex128 vectors
    # (input, output, the Schur part written and read) pass once
    roofp = None
    if calls[4]:
        apply_bytes = 2 * nnz_l * 8 + 16 * 4 * n
        achieved_p = apply_bytes * units[4] / (ms[4] / 1e3) / 1e9
        traffic_p = conv_traffic_from_profile("schur_precon_df_spiral.txt", "dram_bytes_per_rhs_apply")
        roofp = {"kernel": "Schur preconditioner apply (double-float triangular solves, level by level, and the "
                           "SpMVs around them)", "bound": "hbm", "achieved": round(achieved_p, 1), "peak": peak,
                 "unit": "GB/s", "frac": round(achieved_p / peak, 4),
                 "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                 "traffic": round(traffic_p * units[4] / calls[4], 1) if traffic_p else None,
                 "traffic_source": "profiles/schur_precon_df_spiral.txt (ncu, 12-RHS apply, per RHS)",
                 "algorithmic_bytes_per_launch": round(apply_bytes * units[4] / calls[4], 1),
                 "avg_rhs_per_launch": round(units[4] / calls[4], 2), "launches": int(calls[4]),
                 "avg_launch_ms": round(ms[4] / calls[4], 4), "share_of_step_time": round(ms[4] / step_ms_total, 4),
                 "note": "leaf level at 2.5-3 TB/s (partly issue-bound), upper levels latency chains; "
                         "nnz(L) = %d pair entries" % nnz_l}
    # the dominant kernel group of the step is `roofline`; the others follow
    cands = [r for r in ((roofp, ms[4]), (roof32, ms[1]), (roof64, ms[0])) if r[0] is not None]
    cands.sort(key=lambda r: -r[1])
    roof = cands[0][0] if cands else None
    roof_other = [r[0] for r in cands[1:]]
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * t_mixed / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 FFT matvec / f64 Krylov, factor, refinement",
        "data": "synthetic (seeded geometry generator)", "config": cfg,
        "fp64": {"value": round(pts / t_fp64, 4), "ms_per_step": round(1e3 * t_fp64 / args.steps, 3),
                 "dtype": "f64 (complex128 FFT matvec)"},
        "mixed_over_fp64": round(t_fp64 / t_mixed, 3),
        "accuracy": {"reference": "FP64 GPU path converged to GMRES tol 1e-12 (matches the oracle to 1e-9 in tests)",
                     "max_rel_err_R_mixed": err_R, "max_rel_err_L_mixed": err_L,
                     "max_rel_err_R_fp64": err_R64, "max_rel_err_L_fp64": err_L64,
                     "max_rel_err_RL_e2e": err_e2e, "bar": 1e-6,
                     "gmres_iterations_mixed_total": int(it_m.sum()), "gmres_iterations_fp64_total": int(it_d.sum()),
                     "iterations_note": "inner GMRES iterations summed over RHS (mixed: over refinement steps)"},
        "e2e": {"value": round(args.steps * F * world / t_e2e, 4), "unit": UNIT,
                "h2d_bytes_per_step": int(b_host.nbytes + scale.nbytes + 16 * B),
                "d2h_bytes_per_step": int(b_host.nbytes)},
        "gpu_launches": int(launches),
        "sections_ms": sections, "dominant_section": dominant,
        "roofline": roof, "roofline_other": roof_other, "clocks": clk,
    }
    if shared is not None:
        rep_s, t_sh, (R_s, L_s, it_s) = shared
        line["factor_sharing"] = {
            "share_tol": SHARE_TOL, "factors_per_step": int(len(np.unique(rep_s))),
            "value": round(pts / t_sh, 4), "ms_per_step": round(1e3 * t_sh / args.steps, 3),
            "gmres_iterations_total": int(it_s.sum()), "max_rel_err_RL": max(rl_err(R_s, L_s)),
            "note": "mixed path with one Schur factor per group of neighbouring frequencies whose A_inv differs "
                    "by at most share_tol (Sweep.prepare(share_tol)); the headline value factors every frequency"}
    # RHS-matvecs per second of the FFT operator, from the live section timing of the mixed step
    line["matvecs_per_s"] = {
        "complex64": round(sections["fft_conv_c64"]["rhs"] / max(1e-9, sections["fft_conv_c64"]["ms"] / 1e3), 1),
        "double_float": round(sections["fft_conv_df"]["rhs"] / max(1e-9, sections["fft_conv_df"]["ms"] / 1e3), 1),
        "note": "one RHS-matvec = the full operator of lse_matvect_mult.m on one vector; batched calls of ~11 "
                "(complex64) and 32 (refinement residual) vectors"}
    if args.serving_requests >= 0 and world == 1:
        line["serving"] = serving_run(args)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(prob, freqs, sw)
    if rank == 0:
        print(json.dumps(line), flush=True)


def serving_run(args):
    """The serving configuration: the seeded 2000-request stream served in arrival order on this GPU
    (all of it with --serving-requests 2000; by default the first requests up to ~30 s of service),
    latencies under Poisson arrivals at 80 % of the measured capacity."""
    import torch

    from voxhenry_gb300 import serving

    n = args.serving_requests or 2000
    reqs = serving.request_stream(n)
    free, _ = torch.cuda.mem_get_info()
    served = serving.serve(reqs, budget_bytes=int(0.8 * free), max_seconds=None if args.serving_requests else 30.0,
                           min_requests=8)
    out = serving.summarize(served)
    k = out["requests"]
    out["sample"] = (f"the first {k} requests of the seeded 2000-request stream (bars, wires, square spirals; "
                     f"{int(served['freq_points'].sum())} frequency points), mixed precision at GMRES tol 1e-9; "
                     "latency = FIFO queueing under seeded Poisson arrivals + measured service (setup, factors, "
                     "solve, R and L)")
    return out


def _oracle_system(prob):
    """The oracle's System view of a Problem (same arrays; the setup was checked bit-exact)."""
    from oracle import structure as ostruct

    nD = prob.L * prob.M * prob.N
    idxS5 = np.concatenate([prob.idxS + k * nD for k in range(5)])
    return ostruct.System(L=prob.L, M=prob.M, N=prob.N, dx=prob.dx, sigma_e=prob.sigma_e, lambdaL=prob.lambdaL,
                          idxS=prob.idxS, idxS5=idxS5, all_panels_ids=None, num_nodes=prob.meta.get("num_nodes"),
                          Ae_full=None, Ar=prob.Ar, rhs=prob.rhs, nodeid_4_grnd=None, nodeid_4_injectcurr=None,
                          Ae_only_leaving=None, Ae_only_entering_bndry=None)


def cpu_baseline(prob, freqs, sw=None, fN_host=None):
    """The oracle (NumPy/SciPy restatement, FFTs on all host cores) solving ONE frequency point."""
    from oracle import solver
    from voxhenry_gb300 import structure

    if fN_host is None:
        fN_host, st2 = structure.circulant_tensor(prob.L, prob.M, prob.N, prob.dx)
    else:
        fN_host, st2 = fN_host
    S = _oracle_system(prob)
    f = float(freqs[len(freqs) // 2])
    t0 = time.perf_counter()
    out = solver.solve_frequencies(S, fN_host, st2, np.array([f]), restart=RESTART, tol=TOL, maxit=MAXIT)
    t = time.perf_counter() - t0
    return {"value": round(1.0 / t, 6), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"1 of {len(freqs)} frequency points ({f:.3g} Hz) solved to convergence by the oracle "
                      f"({out['iters'][0][2]} GMRES iterations, {t:.1f} s); FFTs threaded over all host cores"}


# ---------------------------------------------------------------------------------------------- reference
def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle import circulant, solver
    from oracle import structure as ostruct

    w, cfg = workload()
    S = ostruct.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    fN, st2 = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    freqs = w.freqs
    jwmu = 1j * 2 * np.pi * freqs[0] * solver.MU0
    z_real, _ = solver.z_arrays(w.sigma_e, None, 2 * np.pi * freqs[0])
    x = S.rhs[:, 0].astype(np.complex128)
    for _ in range(args.warmup):      # warm-up: one matvec each (FFT plans, page-in)
        solver.lse_matvect_mult(x, jwmu * fN, S.Ar, z_real, None, S.dx, S.idxS5)
    n_timed = max(1, min(args.steps, 2))
    sel = [freqs[(len(freqs) // 2 + i * 7) % len(freqs)] for i in range(n_timed)]
    t0 = time.perf_counter()
    out = solver.solve_frequencies(S, fN, st2, np.array(sel), restart=RESTART, tol=TOL, maxit=MAXIT)
    t = time.perf_counter() - t0
    value = n_timed / t
    sample = (f"{n_timed} of {len(freqs)} frequency points solved to convergence "
              f"(GMRES iterations {[it[2] for it in out['iters']]}, {t:.1f} s)")
    line = {"metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * t / n_timed, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded geometry generator)",
            "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_probe(args):
    """Kernel probe for profilers: a few calls of one operator of the workload's geometry (B RHS)."""
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import _lib, executer, structure

    w, _ = workload()
    prob = structure.problem_from_workload(w)
    sw = executer.Sweep(prob, w.freqs, want_fp32=True)
    g = sw.geom
    lib = g.ctx._lib
    B = args.probe_rhs
    x = torch.randn(B, g.n, 2, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    if args.probe in ("conv32", "conv64", "convdf"):
        prec = _lib.PREC[{"conv32": "fp32", "conv64": "fp64", "convdf": "df"}[args.probe]]
        for _ in range(args.probe_iters):
            _lib.check(lib.vh_matvec_device(g.handle, B, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), None,
                                            None, prec), g.ctx.handle)
    else:
        st = (1j * 2 * np.pi * w.freqs[:B] * executer.MU0)[:, None] * np.asarray(prob.st2)[None, :]
        pcs = g.precons(st, np.zeros(B, dtype=np.int32), kind=args.probe_kind)
        parr = (C.c_void_p * B)(*[p.handle for p in pcs])
        if args.probe == "gmres":   # one restart cycle of FP64 GMRES (the FP64 Gram-Schmidt kernels)
            tol = np.full(B, 1e-30)
            flag = np.zeros(B, dtype=np.int32)
            it = np.zeros(2 * B, dtype=np.int32)
            nres = np.zeros(B, dtype=np.int32)
            relres = np.zeros(B)
            ip = C.POINTER(C.c_int)
            scale = np.full(B, 1j * 2 * np.pi * w.freqs[0] * executer.MU0)
            for _ in range(args.probe_iters):
                _lib.check(lib.vh_gmres_device(g.handle, B, parr, C.c_void_p(x.data_ptr()), _lib.cview(scale), None,
                                               args.probe_restart, _lib.dptr(tol), 1, 0, _lib.PREC["fp64"],
                                               C.c_void_p(y.data_ptr()), flag.ctypes.data_as(ip), _lib.dptr(relres),
                                               it.ctypes.data_as(ip), None, 0, nres.ctypes.data_as(ip)), g.ctx.handle)
        else:
            for _ in range(args.probe_iters):
                _lib.check(lib.vh_precon_apply_device(g.handle, B, parr, C.c_void_p(x.data_ptr()),
                                                      C.c_void_p(y.data_ptr())), g.ctx.handle)
    g.ctx.synchronize()
    print(json.dumps({"probe": args.probe, "rhs": B, "iters": args.probe_iters, "launches": int(lib.vh_launch_count())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--probe", choices=["conv32", "conv64", "convdf", "precon", "gmres"], default=None,
                    help="profiling aid: run a few calls of one operator instead of the benchmark")
    ap.add_argument("--mixed-only", action="store_true",
                    help="profiling aid: run only the warm-up and timed mixed-precision sweeps, print nothing")
    ap.add_argument("--serving-requests", type=int, default=0,
                    help="serving configuration: requests of the seeded stream to serve (0: the first ~30 s of "
                         "service; -1: skip)")
    ap.add_argument("--share-tol", type=float, default=None,
                    help="share one Schur factor between neighbouring frequencies whose A_inv differs by at most "
                         "this (mixed path); off by default")
    ap.add_argument("--probe-rhs", type=int, default=4)
    ap.add_argument("--probe-iters", type=int, default=3)
    ap.add_argument("--probe-restart", type=int, default=20)
    ap.add_argument("--probe-kind", default="schur_invert", choices=["schur_invert", "schur_invert_df"])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mixed-precon", default=MIXED_PRECON, choices=["schur_invert_df", "schur_invert"],
                    help="Schur factor arithmetic of the mixed-precision path")
    args = ap.parse_args()
    if args.probe:
        run_probe(args)
        return
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist

        if args.impl == "ours":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
