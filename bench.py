"""Benchmark: frequency points per second of the batched VIE sweep on one GB300.

Headline workload (the largest single-GPU configuration, mixed precision): single-turn circular
ring coil on a 512 x 512 x 16 voxel grid (padded FFT grid 1024 x 1024 x 32), 1 um voxels, radius
150 um, 10 x 10 um square cross-section voxelised by a centre-in-ring test, sigma = 5.8e7 S/m, one
port across a 2 um gap, 16 frequencies log-spaced 1 MHz - 20 GHz solved as 16 right-hand sides in
one batch.  A step is one sweep: the Schur-complement factorisation of every frequency plus the
batched Krylov solve and the R, L extraction.  The circulant tensor, Ae and the symbolic analysis
are set up once before the timed region (resident in HBM).

The other configurations are reported under "configs" with the same measurement:
  C1 straight bar 64 x 16 x 16 (0.5 um voxels, 8 frequencies 1 kHz - 10 GHz; plain FP64 at GMRES
     tol 1e-8, restart 50 -- its own settings -- and both paths at the common tolerance);
  C2 square spiral 256 x 256 x 8 (32 frequencies 1 MHz - 20 GHz);
  C3 two parallel bars 128 x 64 x 32, copper and aluminium (2 ports x 16 frequencies 1 kHz - 10 GHz).
Every configuration's R and L (and the current density x) are compared with the oracle's values
committed in tests/golden/config_<workload>.npz (FP64 reference path converged to tol 1e-12).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--configs C1,C2,C3]

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
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

import numpy as np  # noqa: E402

METRIC = "freq-points/s, mixed-prec batched vs plain FP64 on GB300 @1e-6 R,L; p50/p99 lat"
UNIT = "freq-points/s"
# GMRES tolerance of the mixed and the FP64 path: the loosest that keeps R, L and the current density
# within 1e-6 of the oracle's converged values on these workloads (tol 1e-9 leaves 3e-6 in the spiral's
# current density, tol 1e-8 up to ~5e-6 in R, L)
TOL = 1e-10
RESTART = 50
MAXIT = 10
# the mixed path's Schur factor and triangular solves run in double-float (FP32 pairs, ~48 bits) on
# GB300's FP32 pipes; its FP64 refinement residuals set the final accuracy
MIXED_PRECON = "schur_invert_df"
# factor sharing between neighbouring frequencies for the separately reported variant: A_inv (hence S)
# within 1e-4 of the group's factor
SHARE_TOL = 1e-4

CONFIGS = {
    "C1": {"workload": "bar_64x16x16", "own_tol": 1e-8,
           "text": "straight copper bar, grid 64x16x16 (padded FFT grid 128x32x32), voxel 0.5 um, all voxels "
                   "sigma 5.8e7 S/m, port x=0 face to x=end face, 8 freqs 1 kHz-10 GHz log"},
    "C2": {"workload": "square_spiral_256x256x8",
           "text": "square spiral coil, 4 turns, grid 256x256x8 (padded FFT grid 512x512x16), voxel 1 um, "
                   "trace 5 um x 4 voxels, spacing 2 um, sigma 5.8e7 S/m, 1 port, 32 freqs 1 MHz-20 GHz log"},
    "C3": {"workload": "two_bars_128x64x32",
           "text": "two parallel bars 100x10x10 voxels (copper 5.8e7, aluminium 3.5e7 S/m), 20-voxel gap, grid "
                   "128x64x32 (padded FFT grid 256x128x64), voxel 1 um, 2 ports x 16 freqs 1 kHz-10 GHz log"},
    "C4": {"workload": "ring_512x512x16",
           "text": "circular ring coil, radius 150 um, 10x10 um cross-section, grid 512x512x16 (padded FFT grid "
                   "1024x1024x32), voxel 1 um, sigma 5.8e7 S/m, 1 port across a 2 um gap, 16 freqs 1 MHz-20 GHz log"},
}
HEADLINE = "C4"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(cid):
    from voxhenry_gb300 import geometry

    w = geometry.WORKLOADS[CONFIGS[cid]["workload"]]()
    L, M, N = w.shape
    cfg = {
        "workload": CONFIGS[cid]["text"], "config_id": cid, "grid": [L, M, N], "fft_grid": [2 * L, 2 * M, 2 * N],
        "voxels": int((w.sigma_e > 0).sum()), "ports": len(w.pnt_lft), "freqs": len(w.freqs),
        "rhs_per_step": len(w.freqs) * len(w.pnt_lft),
        "gmres": {"tol": TOL, "restart": RESTART, "maxit": MAXIT, "preconditioner": "schur_invert (left)",
                  "schur_factor": {"mixed": "double-float (FP32 pairs)", "fp64": "fp64"}},
        "l2": "inputs larger than L2: per-RHS vectors of n complex128 and the tensor spectrum (>= 7 x 2L x 2M x 2N "
              "values) per step exceed the 129 MB L2 at C2-C4; C1's working set is re-read from L2 (no flush)",
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


def profile_figure(name, key):
    """A per-unit figure (DRAM bytes per RHS-matvec or per RHS-apply) from a committed ncu summary."""
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


def fixture_accuracy(cid, freqs, R, L, X=None, nc=None):
    """Max relative R, L error (and the current density's) against the oracle fixture, at the
    fixture's frequencies; X: the (F*P, n) solutions of the sweep (host), or None."""
    import config_fixtures as cf

    name = CONFIGS[cid]["workload"]
    if not os.path.exists(cf.path(name)):
        return {"reference": f"missing fixture tests/golden/config_{name}.npz"}
    fx = cf.load(name)
    fi = fx["freq_idx"]
    P = int(fx["ports"])

    def err(a, b):   # per frequency, relative to the largest entry of the port matrix
        return float(max(np.abs(a[k] - b[k]).max() / np.abs(b[k]).max() for k in range(b.shape[0])))

    out = {"reference": f"oracle (FP64 reference path, GMRES tol {float(fx['tol']):g}) at {len(fi)} of "
                        f"{len(freqs)} frequencies: tests/golden/config_{name}.npz",
           "max_rel_err_R": err(R[fi], fx["R"]), "max_rel_err_L": err(L[fi], fx["L"])}
    if X is not None:
        rows = np.concatenate([np.arange(k * P, (k + 1) * P) for k in fi])
        d = cf.compare(X[rows], nc, fx)
        out["max_rel_err_current_density"] = d["curr_sketch"]
        out["max_rel_err_potentials"] = d["phi_sketch"]
        out["x_note"] = "relative 2-norm difference of x estimated by a 64-row Gaussian sketch (about +-25 %)"
    return out


# ---------------------------------------------------------------------------------------------- ours
class ConfigRunner:
    """One configuration's device-resident sweep (geometry, RHS, buffers) and its timed steps."""

    def __init__(self, cid, args, world):
        import torch

        from voxhenry_gb300 import _lib, executer, structure

        self.cid, self.args, self.world = cid, args, world
        self.torch, self._lib, self.executer = torch, _lib, executer
        self.w, self.cfg = workload(cid)
        prob = structure.problem_from_workload(self.w)
        self.prob = prob
        self.freqs = self.w.freqs
        self.sw = executer.Sweep(prob, self.freqs, want_fp32=True)
        g = self.g = self.sw.geom
        if not getattr(args, "no_tune", False):   # the mixed path's FFT products (cached on disk)
            t0 = time.perf_counter()
            tuned = self.sw.tune(precs=("fp32", "df"))
            self.cfg["autotune"] = {p: {k: v for k, v in c.items()} for p, c in tuned.items()}
            self.cfg["autotune"]["seconds"] = round(time.perf_counter() - t0, 2)
        self.lib = g.ctx._lib
        self.stream = torch.cuda.ExternalStream(self.lib.vh_ctx_stream(g.ctx.handle))
        F, P = len(self.freqs), prob.num_ports
        self.F, self.P, self.B, self.n = F, P, F * P, g.n
        rhs = prob.rhs.astype(np.complex128)
        self.b_host = np.ascontiguousarray(np.stack([rhs[:, p] for f in range(F) for p in range(P)]))
        self.scale = np.ascontiguousarray(np.repeat(1j * 2 * np.pi * self.freqs * executer.MU0, P))
        self.zsl = np.ascontiguousarray(np.repeat(self.sw.zslot, P).astype(np.int32))
        self.b_dev = torch.from_numpy(self.b_host.view(np.float64)).cuda()
        self.x_dev = torch.empty_like(self.b_dev)
        self.rhs_dev = torch.from_numpy(prob.rhs.astype(np.float64)).cuda()
        self.flag = np.zeros(self.B, dtype=np.int32)
        self.relres = np.zeros(self.B)
        self.iters = np.zeros(2 * self.B, dtype=np.int32)
        self.nres = np.zeros(self.B, dtype=np.int32)
        self.st_all = (1j * 2 * np.pi * self.freqs * executer.MU0)[:, None] * np.asarray(prob.st2)[None, :]
        # entries of the Schur factor (for the preconditioner's algorithmic bytes); also builds the
        # symbolic analysis before the timed region, as the warm-up would
        pc = g.precons(self.st_all[:1], self.sw.zslot[:1], kind=MIXED_PRECON)
        self.nnz_l = int(pc[0].stats()["nnz_factor"])
        pc[0].close()
        self.share_rep = None

    def precon_kind(self, prec):
        return self.args.mixed_precon if prec == "fp32" else "schur_invert"

    def share_groups(self, tol):
        ex = self.executer
        return ex.factor_share_groups([ex.a_inv_classes(self.prob, f) for f in self.freqs], tol)

    def device_step(self, prec, tol=TOL, maxit=MAXIT, rep=None):
        """One sweep with device-resident inputs: factors + batched solve + R, L."""
        torch, _lib, g = self.torch, self._lib, self.g
        F, P, B, n = self.F, self.P, self.B, self.n
        rep = np.arange(F) if rep is None else rep
        reps = np.unique(rep)
        made = g.precons(self.st_all[reps], self.sw.zslot[reps], kind=self.precon_kind(prec))
        by_rep = dict(zip(reps.tolist(), made))
        pcs = [by_rep[int(r)] for r in rep]
        parr = (C.c_void_p * B)(*[pcs[k // P].handle for k in range(B)])
        tv = np.full(B, tol)
        ip = C.POINTER(C.c_int)
        st = self.lib.vh_gmres_device(g.handle, B, parr, C.c_void_p(self.b_dev.data_ptr()), _lib.cview(self.scale),
                                      self.zsl.ctypes.data_as(ip), RESTART, _lib.dptr(tv), maxit, 0, _lib.PREC[prec],
                                      C.c_void_p(self.x_dev.data_ptr()), self.flag.ctypes.data_as(ip),
                                      _lib.dptr(self.relres), self.iters.ctypes.data_as(ip), None, 0,
                                      self.nres.ctypes.data_as(ip))
        _lib.check(st, g.ctx.handle)
        with torch.cuda.stream(self.stream):
            xc = torch.view_as_complex(self.x_dev.view(B, n, 2))
            Y = torch.einsum("bn,np->bp", xc, self.rhs_dev.to(torch.complex128))   # Y(:, p) = sum rhs .* x
            Yh = Y.cpu().numpy().reshape(F, P, P).transpose(0, 2, 1)
        Z = np.linalg.inv(Yh)
        for p in made:
            p.close()
        return np.abs(Z.real), np.abs(Z.imag) / (2 * np.pi * self.freqs)[:, None, None], self.iters[0::2].copy()

    def x_host(self):
        return self.x_dev.cpu().numpy().view(np.complex128).reshape(self.B, self.n)

    def timed(self, prec, steps, warm, profile=False, rep=None, tol=TOL):
        torch, lib = self.torch, self.lib
        for _ in range(warm):
            self.device_step(prec, rep=rep, tol=tol)
        if self.world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        if profile:
            self._lib.check(lib.vh_ctx_profile(self.g.ctx.handle, 1), self.g.ctx.handle)
        l0 = lib.vh_launch_count()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(self.stream)
        t0 = time.perf_counter()
        out = None
        for _ in range(steps):
            out = self.device_step(prec, rep=rep, tol=tol)
        e1.record(self.stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        launches = lib.vh_launch_count() - l0
        prof = None
        if profile:
            ms = np.zeros(7)
            calls = np.zeros(7, dtype=np.int64)
            units = np.zeros(7, dtype=np.int64)
            self._lib.check(lib.vh_ctx_profile_read(self.g.ctx.handle, self._lib.dptr(ms),
                                                    calls.ctypes.data_as(C.POINTER(C.c_int64)),
                                                    units.ctypes.data_as(C.POINTER(C.c_int64)), 7), self.g.ctx.handle)
            self._lib.check(lib.vh_ctx_profile(self.g.ctx.handle, 0), self.g.ctx.handle)
            prof = (ms, calls, units)
        # the host waits for the device inside every step, so device time == wall time of the region
        t = max(e0.elapsed_time(e1) / 1e3, wall)
        if self.world > 1:
            tt = torch.tensor([t], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t = float(tt.item())
        return t, out, launches, prof

    def rooflines(self, prof, step_ms_total):
        """Roofline entries of the kernel groups of the mixed step (section times: CUDA events on the
        library's stream), dominant first."""
        ms, calls, units = prof
        peak, peak_kind = measured_hbm_peak()
        prob, wl = self.prob, CONFIGS[self.cid]["workload"]

        def fft_roofline(sec, s, st, label, prof_name, note):
            if calls[sec] == 0:
                return None
            avg_b = units[sec] / calls[sec]
            per_rhs = fft_algorithmic_bytes_per_rhs(prob.idxS.size, prob.L, prob.M, prob.N, s, st, avg_b)
            achieved = per_rhs * units[sec] / (ms[sec] / 1e3) / 1e9
            traffic = profile_figure(prof_name, "dram_bytes_per_rhs_matvec")
            return {"kernel": label, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                    "traffic": None if traffic is None else round(traffic * avg_b, 1),
                    "traffic_source": f"profiles/{prof_name} (ncu, per RHS-matvec x RHS per launch)",
                    "algorithmic_bytes_per_launch": round(per_rhs * avg_b, 1),
                    "avg_rhs_per_launch": round(avg_b, 2), "launches": int(calls[sec]),
                    "avg_launch_ms": round(ms[sec] / calls[sec], 4),
                    "share_of_step_time": round(ms[sec] / step_ms_total, 4), "note": note}

        r_df = fft_roofline(0, 16, 16, "FFT circulant matvec in double-float (refinement residuals, VH_PREC_DF: all 5 "
                            "passes in pair arithmetic)", f"fft_matvec_df_{wl}.txt",
                            "frac against HBM with the algorithmic bytes of the two-pass pruned model")
        r_c64 = fft_roofline(1, 8, 4, "FFT circulant matvec, complex64 (inner GMRES matvecs; 5 passes, real/imaginary "
                             "tensor: 4 bytes per component)", f"fft_matvec_c64_{wl}.txt",
                             "frac against HBM with the algorithmic bytes of the two-pass pruned model")
        r_p = None
        if calls[4]:
            apply_bytes = 2 * self.nnz_l * 8 + 16 * 4 * self.n
            achieved = apply_bytes * units[4] / (ms[4] / 1e3) / 1e9
            traffic = profile_figure(f"schur_precon_df_{wl}.txt", "dram_bytes_per_rhs_apply")
            r_p = {"kernel": "Schur preconditioner apply (double-float triangular solves and the SpMVs around them)",
                   "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                   "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                   "traffic": round(traffic * units[4] / calls[4], 1) if traffic else None,
                   "traffic_source": f"profiles/schur_precon_df_{wl}.txt (ncu, per RHS-apply x RHS per launch)",
                   "algorithmic_bytes_per_launch": round(apply_bytes * units[4] / calls[4], 1),
                   "avg_rhs_per_launch": round(units[4] / calls[4], 2), "launches": int(calls[4]),
                   "avg_launch_ms": round(ms[4] / calls[4], 4), "share_of_step_time": round(ms[4] / step_ms_total, 4),
                   "note": "per RHS-apply: the pair factor read once per direction (2 x nnz(L) x 8 B) plus four "
                           "complex128 vector passes; nnz(L) = %d" % self.nnz_l}
        cands = [r for r in ((r_p, ms[4]), (r_c64, ms[1]), (r_df, ms[0])) if r[0] is not None]
        cands.sort(key=lambda r: -r[1])
        return [c[0] for c in cands]

    def run(self, steps, warm, fp64_steps, profile=True, clocks=None):
        """Timed mixed and FP64 sweeps plus accuracy against the oracle fixture."""
        args = self.args
        if clocks:
            clocks.start()
        t_m, out_m, launches, prof = self.timed("fp32", steps, warm, profile=profile)
        clk = clocks.stop() if clocks else None
        X_m = self.x_host()
        t_d, out_d, _, _ = self.timed("fp64", fp64_steps, min(warm, 3))
        X_d = self.x_host()
        R_m, L_m, it_m = out_m
        R_d, L_d, it_d = out_d
        pts_m = steps * self.F * self.world
        pts_d = fp64_steps * self.F * self.world
        sections = None
        roofs = []
        if prof is not None:
            ms, calls, units = prof
            sections = {name: {"ms": round(float(ms[i]), 3), "calls": int(calls[i]), "rhs": int(units[i])}
                        for i, name in enumerate(["fft_conv_df", "fft_conv_c64", "incidence_spmv", "schur_factor",
                                                  "precon_apply", "krylov_vectors", "tensor"])}
            roofs = self.rooflines(prof, 1e3 * t_m)
        res = {
            "workload": self.cfg["workload"], "value": round(pts_m / t_m, 4), "unit": UNIT,
            "steps": steps, "warmup": warm, "ms_per_step": round(1e3 * t_m / steps, 3),
            "fp64": {"value": round(pts_d / t_d, 4), "steps": fp64_steps, "ms_per_step": round(1e3 * t_d / fp64_steps, 3),
                     "dtype": "f64 (complex128 FFT matvec, FP64 factor, solves and Krylov)"},
            "mixed_over_fp64": round((pts_m / t_m) / (pts_d / t_d), 3),
            "accuracy": {"mixed": fixture_accuracy(self.cid, self.freqs, R_m, L_m, X_m, self.prob.Ar.shape[1]),
                         "fp64": fixture_accuracy(self.cid, self.freqs, R_d, L_d, X_d, self.prob.Ar.shape[1]),
                         "bar": 1e-6,
                         "gmres_iterations_mixed_total": int(it_m.sum()),
                         "gmres_iterations_fp64_total": int(it_d.sum()),
                         "iterations_note": "inner GMRES iterations summed over RHS (mixed: over refinement steps)"},
            "gpu_launches": int(launches),
        }
        if sections is not None:
            res["sections_ms"] = sections
            res["matvecs_per_s"] = {
                "complex64": round(sections["fft_conv_c64"]["rhs"] / max(1e-9, sections["fft_conv_c64"]["ms"] / 1e3), 1),
                "double_float": round(sections["fft_conv_df"]["rhs"] / max(1e-9, sections["fft_conv_df"]["ms"] / 1e3), 1),
                "note": "one RHS-matvec = the full operator of lse_matvect_mult.m on one vector (section timing of "
                        "the mixed step)"}
            res["roofline"] = roofs[0] if roofs else None
            res["roofline_other"] = roofs[1:]
        if clk is not None:
            res["clocks"] = clk
        own_tol = CONFIGS[self.cid].get("own_tol")
        if own_tol is not None:   # the configuration's own GMRES settings (plain FP64)
            t_o, out_o, _, _ = self.timed("fp64", fp64_steps, 1, tol=own_tol)
            R_o, L_o, it_o = out_o
            res["fp64_own_settings"] = {
                "tol": own_tol, "restart": RESTART, "maxit": MAXIT, "value": round(pts_d / t_o, 4),
                "ms_per_step": round(1e3 * t_o / fp64_steps, 3), "gmres_iterations_total": int(it_o.sum()),
                "accuracy": fixture_accuracy(self.cid, self.freqs, R_o, L_o, self.x_host(), self.prob.Ar.shape[1])}
        if args.share_tol is not None or self.cid == HEADLINE:
            stol = SHARE_TOL if args.share_tol is None else args.share_tol
            rep = self.share_groups(stol)
            t_s, (R_s, L_s, it_s), _, _ = self.timed("fp32", steps, 1, rep=rep)
            res["factor_sharing"] = {
                "share_tol": stol, "factors_per_step": int(len(np.unique(rep))), "value": round(pts_m / t_s, 4),
                "ms_per_step": round(1e3 * t_s / steps, 3), "gmres_iterations_total": int(it_s.sum()),
                "accuracy": fixture_accuracy(self.cid, self.freqs, R_s, L_s),
                "note": "mixed path with one Schur factor per group of neighbouring frequencies whose A_inv differs "
                        "by at most share_tol (Sweep.prepare(share_tol)); the headline factors every frequency"}
        return res

    def e2e(self, steps, warm):
        """The host-buffer C ABI call a user makes (Sweep -> vh_gmres), copies inside the region."""
        sw = self.sw
        sw.pcs = None
        sw.precon_kind = self.precon_kind("fp32")
        for _ in range(warm):
            sw.prepare().solve(restart=RESTART, tol=TOL, maxit=MAXIT, prec="fp32")
        self.torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = None
        for _ in range(steps):
            sw.pcs = None
            # the previous result is released first, as a caller that keeps no earlier sweep does: its
            # page-locked x block then returns to the host cache and is reused instead of pinning anew
            out = None
            out = sw.prepare().solve(restart=RESTART, tol=TOL, maxit=MAXIT, prec="fp32")
        t = time.perf_counter() - t0
        return {"value": round(steps * self.F * self.world / t, 4), "unit": UNIT,
                "h2d_bytes_per_step": int(self.b_host.nbytes + self.scale.nbytes + 16 * self.B),
                "d2h_bytes_per_step": int(self.b_host.nbytes),
                "accuracy": fixture_accuracy(self.cid, self.freqs, out["R"], out["L"])}

    def close(self):
        self.sw.pcs = None
        self.g.close()


def run_ours(args, rank, world):
    import torch

    import __graft_entry__

    __graft_entry__.build()
    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", "0")))
    fp64_steps = max(1, min(args.steps, args.fp64_steps))
    head = ConfigRunner(HEADLINE, args, world)
    if args.mixed_only:      # profiling aid: only the warm-up and timed mixed-precision steps
        head.timed("fp32", args.steps, args.warmup)
        return
    res = head.run(args.steps, args.warmup, fp64_steps, clocks=ClockSampler(0))
    e2e = head.e2e(args.steps, args.warmup)
    cfg = head.cfg
    line = {
        "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 FFT matvec / f64 Krylov, factor, refinement",
        "data": "synthetic (seeded geometry generator)", "config": cfg,
        "fp64": res["fp64"], "mixed_over_fp64": res["mixed_over_fp64"], "accuracy": res["accuracy"],
        "e2e": e2e, "gpu_launches": res["gpu_launches"], "sections_ms": res.get("sections_ms"),
        "roofline": res.get("roofline"), "roofline_other": res.get("roofline_other"), "clocks": res.get("clocks"),
        "matvecs_per_s": res.get("matvecs_per_s"), "factor_sharing": res.get("factor_sharing"),
    }
    n_head, nnz_head, prob_head = head.n, head.nnz_l, head.prob
    head.close()
    del head
    torch.cuda.empty_cache()
    line["configs"] = {}
    for cid in [c for c in args.configs.split(",") if c and c != HEADLINE]:
        r = ConfigRunner(cid, args, world)
        out = r.run(args.other_steps, args.warmup, fp64_steps)
        out["config"] = r.cfg
        line["configs"][cid] = out
        r.close()
        del r
        torch.cuda.empty_cache()
    if args.serving_requests >= 0 and world == 1:
        line["serving"] = serving_run(args)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(prob_head, HEADLINE, samples=1)
    if rank == 0:
        print(json.dumps(line), flush=True)


def serving_run(args):
    """The serving configuration (continuous batching, voxhenry_gb300.serving.Server) on the seeded
    2000-request stream: a calibration sample of the replayed requests served at saturation on one slot
    and on the server's slots (the speed-up of overlapping requests on the device), then the stream's
    first requests arriving as a seeded Poisson process at 80 % of the measured capacity, replayed on the
    wall clock: p50/p99 latency = completion - arrival."""
    from voxhenry_gb300 import serving

    slots = args.serving_slots
    n_cal = args.serving_calibration
    n = args.serving_requests
    # the replayed requests are the stream's first n; the capacity is measured on n_cal of them taken
    # evenly over that range (request sizes drift along the stream, so its head is not representative)
    stream = serving.request_stream(n)
    step = max(1, n // max(1, n_cal))
    cal = stream[::step][:n_cal]
    out = {"slots": slots}
    srv1 = serving.Server(slots=1, tol=TOL)
    t0 = time.perf_counter()
    srv1.run(cal)
    t1 = time.perf_counter() - t0
    srv1.close()
    srv = serving.Server(slots=slots, tol=TOL)
    t0 = time.perf_counter()
    rk = srv.run(cal)
    tk = time.perf_counter() - t0
    pts = sum(r.freq_points for r in rk)
    out["saturation"] = {"requests": n_cal, "freq_points": int(pts),
                         "one_slot_s": round(t1, 3), f"{slots}_slots_s": round(tk, 3),
                         "freq_points_per_s_one_slot": round(pts / t1, 3),
                         "freq_points_per_s": round(pts / tk, 3), "speedup": round(t1 / tk, 3),
                         "max_in_flight": srv.max_in_flight,
                         "all_converged": serving.summarize_run(rk)["all_converged"]}
    rate = 0.8 * n_cal / tk        # requests per second at 80 % of the measured capacity
    arr = serving.poisson_arrivals(len(stream), rate)
    t0 = time.perf_counter()
    rs = srv.run(stream, arr)
    wall = time.perf_counter() - t0
    srv.close()
    summ = serving.summarize_run(rs, wall)
    summ.update({"arrival_rate_per_s": round(rate, 3), "offered_load": 0.8, "wall_s": round(wall, 2),
                 "max_in_flight": srv.max_in_flight})
    out["poisson"] = summ
    out["p50_latency_s"] = summ["p50_latency_s"]
    out["p99_latency_s"] = summ["p99_latency_s"]
    out["freq_points_per_s"] = summ["freq_points_per_s"]
    out["sample"] = (f"requests 0..{n - 1} of the seeded 2000-request stream (bars, wires, square "
                     f"spirals; {summ['freq_points']} frequency points) arriving as a seeded Poisson process at 80 % of "
                     f"the capacity measured on {len(cal)} of them (every {step}th), replayed on the wall clock; "
                     f"mixed precision at "
                     f"GMRES tol {TOL:g}; {slots} slots (library contexts, one CUDA stream each) admitted first come first "
                     "served by device-memory footprint; latency = completion - arrival")
    return out


# ---------------------------------------------------------------------------------------------- CPU
def _oracle_setup(cid):
    """The oracle's own system and circulant tensor of a configuration (untimed set-up)."""
    from oracle import circulant
    from oracle import structure as ostruct

    w, cfg = workload(cid)
    S = ostruct.build_system(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght)
    fN, st2 = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    return w, cfg, S, fN, st2


def _oracle_iterations(cid, nfreq):
    """The oracle's own GMRES iteration counts at every frequency of a configuration at the
    benchmark tolerance (tests/golden/oracle_iterations.npz, written by the oracle), or None."""
    p = os.path.join(ROOT, "tests", "golden", "oracle_iterations.npz")
    try:
        with np.load(p) as z:
            it = z[CONFIGS[cid]["workload"]]
    except (OSError, KeyError):
        return None
    return it if it.shape[0] == nfreq else None


def oracle_point_sample(S, fN, st2, f, tol=TOL, iters=1):
    """Times one bounded sample of the oracle's work at frequency f: the Schur factorisation of
    lse_sparse_precon_prepare.m (SciPy splu) plus `iters` GMRES iterations of pgmres (each one FFT
    matvec of lse_matvect_mult.m, one preconditioner apply and the Gram-Schmidt step).
    Returns (seconds of the factor, seconds per iteration, total seconds)."""
    from oracle import solver

    t0 = time.perf_counter()
    om = 2 * np.pi * f
    z_real, z_imag = solver.z_arrays(S.sigma_e, S.lambdaL, om)
    jwmu = 1j * om * solver.MU0
    fN_f = jwmu * fN
    pc = solver.SparsePrecon("schur_invert").prepare(S.dx, z_real, z_imag, S.idxS, jwmu * st2, S.Ar)
    t1 = time.perf_counter()
    A = lambda J: solver.lse_matvect_mult(J, fN_f, S.Ar, z_real, z_imag, S.dx, S.idxS5)
    b = S.rhs[:, 0].astype(np.complex128)
    r = pc.multiply(b)
    solver.pgmres_iter(A, np.zeros_like(b), r, iters, pc.multiply, None, 0.0)
    t2 = time.perf_counter()
    return t1 - t0, (t2 - t1) / iters, t2 - t0


def cpu_sample(prob, cid, samples=1, setup=None):
    """The oracle (NumPy/SciPy restatement on all host cores) on a bounded sample of the workload:
    the factorisation and one GMRES iteration at one frequency point, extrapolated to the whole sweep
    with the oracle's own iteration counts at every frequency (the factorisation and an iteration cost
    the same at every frequency: one splu of S, one FFT matvec, one preconditioner apply)."""
    w, cfg, S, fN, st2 = setup or _oracle_setup(cid)
    F = len(w.freqs)
    its = _oracle_iterations(cid, F)
    k = F - 1 if its is None else int(np.argmax(its))
    tf, ti, tt = oracle_point_sample(S, fN, st2, w.freqs[k])
    total_its = int(its.sum()) if its is not None else 10 * F
    sweep = F * tf + ti * total_its
    return {"value": round(F / sweep, 6), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"oracle at {w.freqs[k]:.3g} Hz of the headline workload: Schur factorisation ({tf:.1f} s) and 1 "
                      f"GMRES iteration ({ti:.1f} s) timed, extrapolated to the sweep of {F} points with the "
                      f"oracle's own {total_its} iterations over them ("
                      f"{'tests/golden/oracle_iterations.npz' if its is not None else 'assumed 10 per point'}); "
                      f"FFTs threaded over all host cores"}


def run_reference(args, rank, world):
    """The reference arm: the oracle on the headline workload, each step a bounded sample at one
    frequency (the factorisation plus one GMRES iteration), rotating over the sweep's frequencies;
    the point time extrapolates with the oracle's own iteration count at that frequency."""
    if rank != 0:
        return
    from oracle import solver

    t0 = time.perf_counter()
    w, cfg, S, fN, st2 = _oracle_setup(HEADLINE)
    t_setup = time.perf_counter() - t0
    F = len(w.freqs)
    its = _oracle_iterations(HEADLINE, F)
    if its is None:
        print(json.dumps({"impl": "reference", "unavailable": "oracle iteration table "
                          "tests/golden/oracle_iterations.npz missing for the headline workload"}), flush=True)
        return
    order = [(k * 5) % F for k in range(max(args.steps, F))]   # visits every frequency within F steps
    om = 2 * np.pi * w.freqs[0]
    z_real, z_imag = solver.z_arrays(S.sigma_e, S.lambdaL, om)
    x = S.rhs[:, 0].astype(np.complex128)
    for _ in range(args.warmup):   # warm-up: one matvec each (FFT plans, page-in)
        solver.lse_matvect_mult(x, (1j * om * solver.MU0) * fN, S.Ar, z_real, z_imag, S.dx, S.idxS5)
    t_points = []
    t0 = time.perf_counter()
    for s in range(args.steps):
        k = order[s]
        tf, ti, tt = oracle_point_sample(S, fN, st2, w.freqs[k])
        t_points.append(tf + ti * its[k])
    wall = time.perf_counter() - t0
    value = len(t_points) / sum(t_points)
    sample = (f"each step: the oracle's Schur factorisation and 1 GMRES iteration at one of the {F} frequencies "
              f"(rotating: {sorted(set(order[:args.steps]))}), timed; a frequency point = factorisation + the oracle's "
              f"own iteration count there x the per-iteration time (tests/golden/oracle_iterations.npz, GMRES tol "
              f"{TOL:g}, restart {RESTART}); value = points / sum of their times; ms_per_step = the timed sample; "
              f"set-up (system and circulant tensor) {t_setup:.0f} s, untimed")
    line = {"metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * wall / args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded geometry generator)",
            "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "per_point_seconds": {f"{w.freqs[order[s]]:.4g}": round(t, 2) for s, t in enumerate(t_points)}}
    print(json.dumps(line), flush=True)


def run_probe(args):
    """Kernel probe for profilers: a few calls of one operator of a workload's geometry (B RHS)."""
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import _lib, executer, geometry, structure

    if args.probe_workload == "ring_small":   # the ring's kernels on a 256x256x16 grid (radius 75 um)
        w = geometry.ring(L=256, M=256, N=16, radius=75.0)
    else:
        w, _ = workload(args.probe_workload)
    prob = structure.problem_from_workload(w)
    sw = executer.Sweep(prob, w.freqs, want_fp32=True)
    g = sw.geom
    lib = g.ctx._lib
    B = args.probe_rhs
    x = torch.randn(B, g.n, 2, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    if args.probe in ("conv32", "conv64", "convdf"):
        prec = _lib.PREC[{"conv32": "fp32", "conv64": "fp64", "convdf": "df"}[args.probe]]
        if args.probe_tuning:   # y-pass variant, z-pass variant, right-hand sides per launch[, x variant]
            t = [int(v) for v in args.probe_tuning.split(",")] + [0]
            _lib.check(lib.vh_conv_set_tuning(g.handle, prec, t[0], t[1], t[2], t[3]), g.ctx.handle)
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
    ap.add_argument("--probe-workload", default="C2", choices=list(CONFIGS) + ["ring_small"])
    ap.add_argument("--mixed-only", action="store_true",
                    help="profiling aid: run only the warm-up and timed mixed-precision sweeps, print nothing")
    ap.add_argument("--configs", default="C1,C2,C3",
                    help="configurations reported beside the headline (comma-separated; empty: none)")
    ap.add_argument("--other-steps", type=int, default=3, help="timed steps of the other configurations")
    ap.add_argument("--fp64-steps", type=int, default=3, help="timed steps of the plain FP64 path (at most --steps)")
    ap.add_argument("--serving-requests", type=int, default=48,
                    help="serving configuration: requests of the seeded stream replayed with Poisson arrivals "
                         "(-1: skip the serving configuration)")
    ap.add_argument("--serving-calibration", type=int, default=12,
                    help="serving configuration: requests served at saturation to measure the capacity")
    ap.add_argument("--serving-slots", type=int, default=3, help="serving configuration: requests in flight")
    ap.add_argument("--serving-only", action="store_true",
                    help="run only the serving configuration and print its JSON object")
    ap.add_argument("--share-tol", type=float, default=None,
                    help="also report every configuration with one Schur factor per group of neighbouring "
                         "frequencies whose A_inv differs by at most this (mixed path)")
    ap.add_argument("--probe-rhs", type=int, default=4)
    ap.add_argument("--probe-iters", type=int, default=3)
    ap.add_argument("--probe-restart", type=int, default=20)
    ap.add_argument("--probe-tuning", default=None,
                    help="conv probes: 'y,z,max_rhs[,x]' as vh_conv_set_tuning takes them (default: untuned)")
    ap.add_argument("--probe-kind", default="schur_invert", choices=["schur_invert", "schur_invert_df"])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the FFT convolution's default launch choices")
    ap.add_argument("--mixed-precon", default=MIXED_PRECON, choices=["schur_invert_df", "schur_invert"],
                    help="Schur factor arithmetic of the mixed-precision path")
    args = ap.parse_args()
    if args.probe:
        run_probe(args)
        return
    if args.serving_only:
        import __graft_entry__

        __graft_entry__.build()
        print(json.dumps(serving_run(args)), flush=True)
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
