"""Oracle: FFT matvec, Schur preconditioner, (F)GMRES and the executer loop (test infrastructure).

Restates:
  * src_lse_formation/lse_matvect_mult.m:1-140           -> lse_matvect_mult
  * src_lse_formation/lse_sparse_precon_prepare.m:33-102  -> SparsePrecon.prepare (schur_invert; SuperLU
    in place of CHOLMOD ldlchol, i.e. the Octave lu path :12-15, 123-126)
  * src_lse_formation/lse_sparse_precon_multiply.m:61-117 -> SparsePrecon.multiply
  * src_iterative_solver/pgmres.m:70-198, pgmres_iter.m:22-153 -> pgmres
  * src_iterative_solver/fpgmres.m:58-153, fpgmres_iter.m     -> fpgmres
  * VoxHenry_executer.m:215-329                            -> solve_frequencies
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.fft as sfft
import scipy.sparse as sp
import scipy.sparse.linalg as spla

MU0 = 4 * np.pi * 1e-7          # EMconstants.m:13
WORKERS = os.cpu_count() or 1   # FFTs threaded over the host cores (MATLAB's fftn is multithreaded)
DIAG_SCALE = np.array([1.0, 1.0, 1.0, 1.0 / 6.0, 1.0 / 2.0])   # lse_matvect_mult.m:99-103


def _tensor_products(G, F):
    """The five output spectra of lse_matvect_mult.m:57-93 from the five input spectra F and the seven
    tensor components G, element by element in the reference's order of operations; ranges of the
    grid run on all host cores (numpy releases the GIL inside the array operations)."""
    shape = F[0].shape
    n = F[0].size
    Gf = [g.reshape(-1, order="F") for g in G]
    Ff = [f.reshape(-1, order="F") for f in F]
    out = [np.empty(n, dtype=np.complex128) for _ in range(5)]

    def part(a, b):
        g = [x[a:b] for x in Gf]
        f = [x[a:b] for x in Ff]
        J1 = g[0] * f[0]
        J4 = -g[1] * f[0]
        J5 = J4.copy()
        J2 = g[0] * f[1]
        J4 = J4 - g[2] * f[1]
        J5 = J5 + g[2] * f[1]
        J3 = g[0] * f[2]
        J5 = J5 - g[4] * f[2]
        J1 = J1 + g[1] * f[3]
        J2 = J2 + g[2] * f[3]
        J4 = J4 + g[3] * f[3]
        J5 = J5 + g[5] * f[3]
        J1 = J1 + g[1] * f[4]
        J2 = J2 - g[2] * f[4]
        J3 = J3 + g[4] * f[4]
        J4 = J4 + g[5] * f[4]
        J5 = J5 + g[6] * f[4]
        for o, J in zip(out, (J1, J2, J3, J4, J5)):
            o[a:b] = J

    step = max(1 << 16, -(-n // (4 * WORKERS)))
    with ThreadPoolExecutor(max_workers=WORKERS) as ex:
        list(ex.map(lambda a: part(a, min(n, a + step)), range(0, n, step)))
    return [o.reshape(shape, order="F") for o in out]


def lse_matvect_mult(JIn0, fN_all, Ae, z_real, z_imag, dx, idx):
    """lse_matvect_mult.m:1-140 (fl_precon_type != 'schur_invert_original')."""
    num_node, num_curr = Ae.shape
    LfN, MfN, NfN, _ = fN_all.shape
    L, M, N = z_real.shape
    JIn = np.zeros(L * M * N * 5, dtype=np.complex128)
    JIn[idx - 1] = JIn0[:num_curr]
    JIn = JIn.reshape(L, M, N, 5, order="F")
    F = [sfft.fftn(JIn[:, :, :, c], s=(LfN, MfN, NfN), workers=WORKERS) for c in range(5)]
    G = [fN_all[:, :, :, k] for k in range(7)]
    Js = _tensor_products(G, F)
    del F
    outs = [sfft.ifftn(J, workers=WORKERS) for J in Js]
    zz = z_real if z_imag is None else (z_real + z_imag)
    JOut = np.zeros((L, M, N, 5), dtype=np.complex128, order="F")
    with np.errstate(invalid="ignore"):
        for c in range(5):
            JOut[:, :, :, c] = (DIAG_SCALE[c] / dx) * zz * JIn[:, :, :, c] + outs[c][:L, :M, :N]
    JOut = JOut.reshape(-1, order="F")[idx - 1]
    out = np.zeros(num_curr + num_node, dtype=np.complex128)
    out[:num_curr] = JOut - Ae.T @ JIn0[num_curr:num_curr + num_node]
    out[num_curr:] = Ae @ JIn0[:num_curr]
    return out


def z_arrays(sigma_e, lambdaL, omega):
    """VoxHenry_executer.m:231-259: (z_real, z_imag or None)."""
    if lambdaL is None:
        with np.errstate(divide="ignore"):
            return 1.0 / sigma_e, None
    mu = MU0
    den = (omega * mu * sigma_e * lambdaL**2) ** 2 + 1
    z_real = (sigma_e * (omega * mu * lambdaL**2) ** 2) / den
    z_imag = (1j * omega * mu * lambdaL**2) / den
    sig_nz = np.abs(sigma_e) > 1e-12
    lam_nz = np.abs(lambdaL) > 1e-12
    sel = (~lam_nz) & sig_nz
    with np.errstate(divide="ignore"):
        inv = 1.0 / sigma_e
    z_real = np.where(sel, inv, z_real)
    z_imag = np.where(sel, 0.0, z_imag)
    return z_real, z_imag


def a_inv_diag(dx, z_real, z_imag, idxS, st):
    """lse_sparse_precon_prepare.m:36-62: the real diagonal |1/(z/(c dx) + st_k)|, length 5 Nv."""
    zr = z_real.reshape(-1, order="F")[idxS - 1]
    zz = zr if z_imag is None else zr + z_imag.reshape(-1, order="F")[idxS - 1]
    d_pulse = 1.0 / (zz / dx + st[0])
    d_2d = 1.0 / (zz / (6 * dx) + st[1])
    d_3d = 1.0 / (zz / (2 * dx) + st[2])
    return np.abs(np.concatenate([d_pulse, d_pulse, d_pulse, d_2d, d_3d]))


class SparsePrecon:
    """State of lse_sparse_precon_prepare / lse_sparse_precon_multiply (MATLAB globals)."""

    def __init__(self, kind: str = "schur_invert"):
        self.kind = kind

    def prepare(self, dx, z_real, z_imag, idxS, st, Ae):
        if self.kind == "no_precond":
            return self
        self.Ae = sp.csr_matrix(Ae)
        self.AeT = sp.csr_matrix(Ae.T)
        self.A_inv = a_inv_diag(dx, z_real, z_imag, idxS, st)
        if self.kind == "schur_invert":
            S = (self.Ae @ sp.diags(self.A_inv) @ self.AeT).tocsc()
            self.S = S
            # symmetric-mode SuperLU with a minimum-degree ordering of S + S^T
            self.lu = spla.splu(S, permc_spec="MMD_AT_PLUS_A", options=dict(SymmetricMode=True))
        elif self.kind == "schur_approx":
            # prepare.m:71-81: A_noninv = inv(A_inv), W = diag(1 / sum(|Ae|, 2))
            self.A_noninv = 1.0 / self.A_inv
            w = np.asarray(abs(self.Ae).sum(axis=1)).ravel()
            self.Wd = 1.0 / w
        elif self.kind == "schur_gmres":
            # prepare.m:83-88: S = Ae A_inv Ae', precond = diag(S); S v by lse_sparse_schur_compl_multiply.m:3
            self.S = (self.Ae @ sp.diags(self.A_inv) @ self.AeT).tocsr()
            self.Sd = self.S.diagonal()
            self.prectol = 0.1            # VoxHenry_executer.m:38
            self.inner_iters = 0
        else:
            raise NotImplementedError(self.kind)
        return self

    def schur_gmres_solve(self, bb):
        """multiply.m:43: gmres(fPSchur, bb, min(100, num_curr - 1), prectol, 10, precond).

        The inner solver is MATLAB's built-in gmres (not part of the reference's sources).  Restated from
        its published algorithm: restarted GMRES (Saad & Schultz 1986) with x0 = 0 and the left
        preconditioner M = precond = diag(S), stopping when the preconditioned relative residual
        |M^-1 (bb - S x)| / |M^-1 bb| <= prectol; a zero right-hand side gives x = 0.  The restatement
        orthogonalises by classical Gram-Schmidt (the oracle's pgmres) where MATLAB uses Householder
        reflections: the same Krylov minimiser in exact arithmetic."""
        if not np.any(bb):
            return np.zeros_like(bb)
        nc = self.Ae.shape[1]
        x, _, _, _, resvec = pgmres(lambda v: self.S @ v, bb, restart=min(100, nc - 1), tol=self.prectol,
                                    maxit=10, L1=lambda v: v / self.Sd)
        self.inner_iters += len(resvec) - 1
        return x

    def solve_S(self, b):
        # the factor is real; apply it to the real and imaginary parts
        if np.iscomplexobj(b):
            return self.lu.solve(np.ascontiguousarray(b.real)) + 1j * self.lu.solve(np.ascontiguousarray(b.imag))
        return self.lu.solve(b)

    def multiply(self, x):
        """lse_sparse_precon_multiply.m:61-117 (schur_invert), :48-58 (schur_approx), :26-46 (schur_gmres)."""
        if self.kind == "no_precond":
            return x.copy()
        nc = self.Ae.shape[1]
        a = x[:nc]
        b = x[nc:]
        out = np.zeros_like(x)
        bb = b - self.Ae @ (self.A_inv * a)
        if self.kind == "schur_invert":
            out[nc:] = self.solve_S(bb)
        elif self.kind == "schur_gmres":
            out[nc:] = self.schur_gmres_solve(bb)
        else:
            t = self.AeT @ (self.Wd * bb)
            out[nc:] = self.Wd * (self.Ae @ (self.A_noninv * t))
        out[:nc] = (a - (-(self.AeT @ out[nc:]))) * self.A_inv
        return out


def _apply(op, x):
    if op is None:
        return x
    if callable(op):
        return op(x)
    return spla.spsolve(op, x) if sp.issparse(op) else np.linalg.solve(op, x)


def pgmres_iter(A, x, r, m, L1, R1, tol):
    """pgmres_iter.m:22-153 (one left and one right preconditioner, as the executer uses)."""
    n = r.size
    V = np.zeros((n, m + 1), dtype=np.complex128)
    rnorm = np.linalg.norm(r)
    V[:, 0] = r / rnorm
    H = np.zeros((m + 1, m), dtype=np.complex128)
    resvec = np.zeros(m)
    y = None
    res = None
    k = 0
    for k in range(1, m + 1):
        w = V[:, k - 1]
        if R1 is not None:
            w = _apply(R1, w)
        w = A(w)
        if L1 is not None:
            w = _apply(L1, w)
        h = V[:, :k].conj().T @ w                      # classical Gram-Schmidt (:107-108)
        w = w - V[:, :k] @ h
        H[:k, k - 1] = h
        H[k, k - 1] = np.linalg.norm(w)
        V[:, k] = w / H[k, k - 1]
        rhs = np.zeros(k + 1, dtype=np.complex128)
        rhs[0] = rnorm
        Hc = H[: k + 1, :k]
        y = np.linalg.lstsq(Hc, rhs, rcond=None)[0]    # Hc \ rhs (:118-119)
        res = rhs - Hc @ y
        resvec[k - 1] = np.linalg.norm(res)
        if resvec[k - 1] < tol:
            break
    xupd = V[:, :k] @ y
    if R1 is not None:
        xupd = _apply(R1, xupd)
    return x + xupd, V[:, : k + 1] @ res, k, resvec[:k]


def pgmres(A, b, restart=50, tol=1e-3, maxit=10, L1=None, R1=None, x0=None):
    """pgmres.m:70-198 -> (x, flag, relres, iter, resvec)."""
    x = np.zeros_like(b, dtype=np.complex128) if x0 is None else x0.astype(np.complex128)
    r = b - A(x) if np.count_nonzero(x) else b.astype(np.complex128)
    bp = b.astype(np.complex128)
    if L1 is not None:
        r = _apply(L1, r)
        bp = _apply(L1, bp)
    bnorm = np.linalg.norm(bp)
    resvec = [np.linalg.norm(r) / bnorm]
    outit = 0
    p = 0
    while resvec[-1] > tol and outit < maxit:
        outit += 1
        x, r, p, rin = pgmres_iter(A, x, r, restart, L1, R1, tol * bnorm)
        resvec.extend(list(rin / bnorm))
    relres = np.linalg.norm(b - A(x)) / np.linalg.norm(b)
    flag = 0 if relres <= tol else 1
    return x, flag, relres, (p, outit), np.array(resvec)


def fpgmres_iter(A, x, r, m, R1, tol):
    """fpgmres_iter.m: flexible GMRES, right preconditioner, stores Z."""
    n = r.size
    V = np.zeros((n, m + 1), dtype=np.complex128)
    Z = np.zeros((n, m), dtype=np.complex128)
    rnorm = np.linalg.norm(r)
    V[:, 0] = r / rnorm
    H = np.zeros((m + 1, m), dtype=np.complex128)
    resvec = np.zeros(m)
    k = 0
    for k in range(1, m + 1):
        Z[:, k - 1] = V[:, k - 1] if R1 is None else _apply(R1, V[:, k - 1])
        w = A(Z[:, k - 1])
        h = V[:, :k].conj().T @ w
        w = w - V[:, :k] @ h
        H[:k, k - 1] = h
        H[k, k - 1] = np.linalg.norm(w)
        V[:, k] = w / H[k, k - 1]
        rhs = np.zeros(k + 1, dtype=np.complex128)
        rhs[0] = rnorm
        Hc = H[: k + 1, :k]
        y = np.linalg.lstsq(Hc, rhs, rcond=None)[0]
        res = rhs - Hc @ y
        resvec[k - 1] = np.linalg.norm(res)
        if resvec[k - 1] < tol:
            break
    return x + Z[:, :k] @ y, V[:, : k + 1] @ res, k, resvec[:k]


def fpgmres(A, b, restart=50, tol=1e-3, maxit=10, R1=None, x0=None):
    """fpgmres.m:58-153 -> (x, flag, relres, iter, resvec)."""
    x = np.zeros_like(b, dtype=np.complex128) if x0 is None else x0.astype(np.complex128)
    r = b - A(x) if np.count_nonzero(x) else b.astype(np.complex128)
    bnorm = np.linalg.norm(b)
    resvec = [np.linalg.norm(r) / bnorm]
    outit = 0
    p = 0
    while resvec[-1] > tol and outit < maxit:
        outit += 1
        x, r, p, rin = fpgmres_iter(A, x, r, restart, R1, tol * bnorm)
        resvec.extend(list(rin / bnorm))
    relres = np.linalg.norm(b - A(x)) / np.linalg.norm(b)
    flag = 0 if relres <= tol else 1
    return x, flag, relres, (p, outit), np.array(resvec)


def solve_frequencies(sysm, fN_all2, st2, freqs, restart=100, maxit=10, tol=None,
                      precon="schur_invert", keep_x=False):
    """VoxHenry_executer.m:215-329 -> dict with Y, Z, R, L per frequency (and x if asked).

    ``tol=None`` applies the executer's rule (1e-12 below 1 MHz, else 1e-8).
    """
    nf = len(freqs)
    P = sysm.rhs.shape[1]
    Y = np.zeros((nf, P, P), dtype=np.complex128)
    xs, iters = [], []
    for fi, f in enumerate(freqs):
        t = (1e-12 if f < 1e6 else 1e-8) if tol is None else tol
        omega = 2 * np.pi * f
        z_real, z_imag = z_arrays(sysm.sigma_e, sysm.lambdaL, omega)
        jwmu = 1j * omega * MU0
        fN = jwmu * fN_all2
        st = jwmu * st2
        pc = SparsePrecon(precon).prepare(sysm.dx, z_real, z_imag, sysm.idxS, st, sysm.Ar)
        A = lambda J: lse_matvect_mult(J, fN, sysm.Ar, z_real, z_imag, sysm.dx, sysm.idxS5)
        for p in range(P):
            b = sysm.rhs[:, p].astype(np.complex128)
            if precon == "schur_gmres":   # VoxHenry_executer.m:294-297: the flexible solver
                x, flag, relres, it, resvec = fpgmres(A, b, restart, t, maxit, pc.multiply)
            else:
                x, flag, relres, it, resvec = pgmres(A, b, restart, t, maxit, pc.multiply)
            Y[fi, :, p] = sysm.rhs.T @ x                  # sum(rhs(:,kk).*x), no conjugate
            iters.append((f, p, len(resvec) - 1, relres))
            if keep_x:
                xs.append(x)
    Z = np.linalg.inv(Y)
    R = np.abs(Z.real)
    Lh = np.abs(Z.imag) / (2 * np.pi * np.asarray(freqs))[:, None, None]
    out = {"Y": Y, "Z": Z, "R": R, "L": Lh, "iters": iters}
    if keep_x:
        out["x"] = xs
    return out
