"""Batched frequency sweep of VoxHenry_executer.m:215-329 on the GPU.

All frequencies and ports of a job are solved as one batch of right-hand sides: one FFT
matvec call per Krylov step for the whole batch (the tensor spectrum fN_all2 is shared, each RHS
carries its own j*omega*mu), one Schur-complement factor per frequency (shared by the ports of
that frequency), one Krylov space per RHS.  Y(:, p) = sum(rhs .* x) (no conjugate,
VoxHenry_executer.m:311-316), Z = inv(Y), R = |Re Z|, L = |Im Z| / (2 pi f) (:327-328).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

from . import _lib, vie

MU0 = 4 * np.pi * 1e-7     # EMconstants.m:13


@dataclass
class Problem:
    """Inputs of the solve loop (the executer's state after VoxHenry_executer.m:200)."""
    L: int
    M: int
    N: int
    dx: float
    sigma_e: np.ndarray               # (L, M, N)
    lambdaL: np.ndarray | None
    idxS: np.ndarray                  # 1-based
    Ar: sp.csc_matrix                 # Ae with port rows removed
    rhs: np.ndarray                   # (n, num_ports) real
    fN_all2: np.ndarray               # (2L, 2M, 2N, 7) complex, without j*omega*mu
    st2: np.ndarray                   # (3,) complex self terms, without j*omega*mu
    meta: dict = field(default_factory=dict)

    @property
    def num_ports(self):
        return self.rhs.shape[1]


def z_arrays(sigma_e, lambdaL, omega):
    """VoxHenry_executer.m:231-259 -> (z_real, z_imag or None)."""
    if lambdaL is None:
        with np.errstate(divide="ignore"):
            return 1.0 / sigma_e, None
    den = (omega * MU0 * sigma_e * lambdaL**2) ** 2 + 1
    z_real = (sigma_e * (omega * MU0 * lambdaL**2) ** 2) / den
    z_imag = (1j * omega * MU0 * lambdaL**2) / den
    sel = (np.abs(lambdaL) <= 1e-12) & (np.abs(sigma_e) > 1e-12)
    with np.errstate(divide="ignore"):
        inv = 1.0 / sigma_e
    return np.where(sel, inv, z_real), np.where(sel, 0.0, z_imag)


def executer_tol(f: float) -> float:
    """VoxHenry_executer.m:219-223."""
    return 1e-12 if f < 1e6 else 1e-8


def a_inv_classes(prob: Problem, f: float) -> np.ndarray:
    """The diagonal A_inv of lse_sparse_precon_prepare.m:33-64 at frequency f, (nv, 3) for the
    Jx/Jy/Jz, J2D and J3D classes (host copy, used to decide factor sharing)."""
    om = 2 * np.pi * f
    idx = np.asarray(prob.idxS).ravel() - 1
    sig = np.asarray(prob.sigma_e).ravel(order="F")[idx]
    lam = None if prob.lambdaL is None else np.asarray(prob.lambdaL).ravel(order="F")[idx]
    zr, zi = z_arrays(sig, lam, om)            # elementwise: evaluated on the voxels only
    z = zr + (0 if zi is None else zi)
    st = 1j * om * MU0 * np.asarray(prob.st2)
    dx = prob.dx
    return np.abs(1.0 / np.stack([z / dx + st[0], z / (6 * dx) + st[1], z / (2 * dx) + st[2]], axis=1))


def factor_share_groups(a_invs, share_tol: float) -> np.ndarray:
    """Groups of consecutive frequencies that share one Schur factor: a frequency joins the current
    group while its A_inv differs from the group's first by at most share_tol (max relative change);
    returns the representative frequency index of each frequency."""
    rep = np.zeros(len(a_invs), dtype=np.int64)
    r = 0
    for i in range(1, len(a_invs)):
        if np.max(np.abs(a_invs[i] - a_invs[r]) / a_invs[r]) > share_tol:
            r = i
        rep[i] = r
    return rep


class Sweep:
    """Device-resident job: geometry (tensor, Ae, z slots) plus one factor per frequency."""

    def __init__(self, prob: Problem, freqs, want_fp32=True, precon="schur_invert", ctx=None):
        self.prob = prob
        self.freqs = np.asarray(freqs, dtype=np.float64)
        t0 = time.perf_counter()
        z0, zi0 = z_arrays(prob.sigma_e, prob.lambdaL, 2 * np.pi * self.freqs[0])
        if prob.fN_all2 is None:     # tensor generated on the device (lse_generate_circulant_tensor)
            self.geom, prob.st2 = vie.Geometry.generated(prob.L, prob.M, prob.N, prob.dx, prob.Ar, z0, zi0, prob.idxS,
                                                         want_fp32=want_fp32, ctx=ctx)
        else:
            self.geom = vie.Geometry(prob.fN_all2, prob.Ar, z0, zi0, prob.dx, prob.idxS, want_fp32=want_fp32, ctx=ctx)
        self.super = prob.lambdaL is not None
        self.zslot = np.zeros(len(self.freqs), dtype=np.int32)
        if self.super:                                   # omega-dependent z: one slot per frequency
            for i, f in enumerate(self.freqs):
                zr, zi = z_arrays(prob.sigma_e, prob.lambdaL, 2 * np.pi * f)
                self.geom.set_z(i, zr, zi)
                self.zslot[i] = i
        self.t_setup = time.perf_counter() - t0
        self.precon_kind = precon
        self.pcs = None
        self.t_factor = 0.0

    def set_frequencies(self, freqs):
        """Solves another frequency list on the same resident geometry (tensor, Ae, symbolic analysis);
        superconductors get their z slots for the new frequencies."""
        self.freqs = np.asarray(freqs, dtype=np.float64)
        self.zslot = np.zeros(len(self.freqs), dtype=np.int32)
        if self.super:
            for i, f in enumerate(self.freqs):
                zr, zi = z_arrays(self.prob.sigma_e, self.prob.lambdaL, 2 * np.pi * f)
                self.geom.set_z(i, zr, zi)
                self.zslot[i] = i
        self.pcs = None
        self.__dict__.pop("_b_host", None)
        self.__dict__.pop("_share_groups", None)
        return self

    def tune(self, precs=("fp32", "df"), path: str | None = None, retune: bool = False) -> dict:
        """Autotunes the FFT convolution for this sweep's batch (all frequencies x ports) at each
        precision (voxhenry_gb300.autotune; cached on disk)."""
        from . import autotune

        B = len(self.freqs) * self.prob.num_ports
        grid = (self.prob.L, self.prob.M, self.prob.N)
        box = autotune.box_of(self.prob)
        return {p: autotune.tune(self.geom, p, B, grid, box, path=path, retune=retune) for p in precs}

    def prepare(self, share_tol: float | None = None):
        """lse_sparse_precon_prepare for every frequency (VoxHenry_executer.m:273).

        share_tol (not in the reference, off by default): neighbouring frequencies whose A_inv differs
        by at most share_tol use one factor (the preconditioner of the group's first frequency).  The
        solution still converges to tol; only the iteration count can change, since S is linear in
        A_inv and the shared factor is S's within share_tol."""
        t0 = time.perf_counter()
        jwmu = 1j * 2 * np.pi * self.freqs * MU0
        st = jwmu[:, None] * np.asarray(self.prob.st2)[None, :]
        if share_tol is None:
            self.factor_of = np.arange(len(self.freqs))
            self.pcs = self.geom.precons(st, self.zslot, kind=self.precon_kind)
        else:
            cache = self.__dict__.setdefault("_share_groups", {})
            if share_tol not in cache:   # the frequencies of a sweep are fixed: group them once
                cache[share_tol] = factor_share_groups([a_inv_classes(self.prob, f) for f in self.freqs], share_tol)
            self.factor_of = cache[share_tol]
            reps = np.unique(self.factor_of)
            made = self.geom.precons(st[reps], self.zslot[reps], kind=self.precon_kind)
            by_rep = dict(zip(reps.tolist(), made))
            self.pcs = [by_rep[int(r)] for r in self.factor_of]
        self.t_factor = time.perf_counter() - t0
        return self

    def _rhs_batch(self) -> np.ndarray:
        """The (F * P, n) right-hand sides, frequency-major (rhs(:, p) for every frequency), built once
        per sweep in page-locked host memory; the solve copies it to the device on every call."""
        b = self.__dict__.get("_b_host")
        if b is None:
            P, F = self.prob.num_ports, len(self.freqs)
            b = _lib.host_empty((F * P, self.geom.n), np.complex128)
            rhs = self.prob.rhs.astype(np.complex128)
            for fi in range(F):
                b[fi * P:(fi + 1) * P] = rhs.T
            self._b_host = b
        return b

    def solve(self, restart=50, tol=None, maxit=10, prec="fp64", flexible=False):
        """Solves every (frequency, port) RHS in one batch; returns R, L, Y, Z and solver stats."""
        if self.pcs is None:
            self.prepare()
        P = self.prob.num_ports
        F = len(self.freqs)
        B = F * P
        b = self._rhs_batch()
        scale = np.empty(B, dtype=np.complex128)
        zsl = np.empty(B, dtype=np.int32)
        tolv = np.empty(B)
        pcs = []
        for fi, f in enumerate(self.freqs):
            for p in range(P):
                k = fi * P + p
                scale[k] = 1j * 2 * np.pi * f * MU0
                zsl[k] = self.zslot[fi]
                tolv[k] = executer_tol(f) if tol is None else tol
                pcs.append(self.pcs[fi])
        # the 'schur_gmres' apply is an inner iterative solve: flexible GMRES (VoxHenry_executer.m:294-297)
        flexible = flexible or self.precon_kind == "schur_gmres"
        t0 = time.perf_counter()
        out = self.geom.solve(b, pcs=pcs, scale=scale, zslot=zsl, restart=restart, tol=tolv, maxit=maxit,
                              flexible=flexible, prec=prec)
        t_solve = time.perf_counter() - t0
        x = out["x"]
        # Y(:, p) = sum(rhs .* x) (VoxHenry_executer.m:311-316); rhs is nonzero only on the port rows
        rows = np.flatnonzero(np.any(self.prob.rhs != 0, axis=1))
        Yall = x[:, rows] @ self.prob.rhs[rows]   # (B, P): Yall[k, q] = sum_n rhs[n, q] x_k[n]
        Y = Yall.reshape(F, P, P).transpose(0, 2, 1).copy()
        Z = np.linalg.inv(Y)
        R = np.abs(Z.real)
        Lh = np.abs(Z.imag) / (2 * np.pi * self.freqs)[:, None, None]
        return {"R": R, "L": Lh, "Y": Y, "Z": Z, "x": x, "flag": out["flag"], "relres": out["relres"],
                "iter": out["iter"], "resvec": out["resvec"], "t_solve": t_solve, "t_factor": self.t_factor}
