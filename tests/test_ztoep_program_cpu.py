"""The Toeplitz z-pass's warp program against the oracle's tensor products along one (kx, ky) column.

`k_zpass_toep` and `k_zpass_toep_df` (voxhenry_gb300/csrc/vh_conv_ztoep.cu) split the 13 distinct
convolutions of the operator over five warps by a constant step table, `kZtProgram`: per step a body
kind (even kernel, combined inputs times i, odd kernel), a kernel index and the inputs.  This test
reads that table from the source and runs it in NumPy the way the kernels do (the partial sums A, B
and P of warps 0-2 first, rotated by i for the imaginary kernels of the complex64 pass, then the
hand-off to warps 3-4), on random kernels of each symmetry class the table builder admits (real even:
G0, G3, G5, G6; imaginary even: G1, G2; real odd: G4).  The reference is the oracle's spectral product
(`_tensor_products`, lse_matvect_mult.m:57-93) on the column's z spectra with the inputs zero-padded
to a linear-convolution length, which is what the z FFT pair computes."""
import os
import re

import numpy as np
import pytest

from oracle import solver

SRC = os.path.join(os.path.dirname(__file__), "..", "voxhenry_gb300", "csrc", "vh_conv_ztoep.cu")
IMAG = {1, 2}
ODD = {4}


def program():
    s = open(SRC).read()
    body = s[s.index("kZtProgram[5][3] = {"):]
    body = body[body.index("{") + 1:body.index("};")]
    rows = re.findall(r"\{([^{}]*)\}", body)
    out = []
    for r in rows:
        codes = []
        for e in r.split(","):
            e = e.strip()
            assert re.fullmatch(r"[0-9 |<]+", e), e   # integer constants, | and << only
            codes.append(eval(e, {"__builtins__": {}}))
        out.append(codes)
    assert len(out) == 5 and all(len(c) == 3 for c in out)
    return out


def decode(code):
    return code & 3, (code >> 2) & 7, (code >> 5) & 7, (code >> 8) & 7, (code >> 11) & 1


def kernels(rng, nz):
    """g_k[d], d < nz: the real table values (imaginary kernels: h = i g; odd: h(-d) = -h(d), g[0] = 0)."""
    g = rng.standard_normal((7, nz))
    g[4, 0] = 0.0
    return g


def h_two_sided(g, k, d):
    v = g[k][abs(d)]
    if d < 0 and k in ODD:
        v = -v
    return 1j * v if k in IMAG else v


def toeplitz(g, k, nz, real_body):
    """The matrix of kernel k on nz rows; real_body: the table values without the factor i."""
    T = np.zeros((nz, nz), complex)
    for m in range(nz):
        for n in range(nz):
            h = h_two_sided(g, k, m - n)
            T[m, n] = h / 1j if (real_body and k in IMAG) else h
    return T


def run_c64(prog, g, j):
    """k_zpass_toep: bodies by kind, kernels as stored (imaginary ones without i); A and B rotated."""
    nz = j.shape[1]
    part, out = [None] * 3, [None] * 5
    for w in range(5):
        acc = np.zeros(nz, complex)
        for st in range(0 if w < 3 else 1, 3):
            kind, k, c1, c2, neg = decode(prog[w][st])
            T = toeplitz(g, k, nz, real_body=True)
            if kind == 1:
                acc = acc + 1j * (T @ (j[c1] + (-1.0 if neg else 1.0) * j[c2]))
            else:
                assert (kind == 2) == (k in ODD), (w, st)
                acc = acc + T @ j[c1]
            if st == 0:
                part[w] = 1j * acc if w < 2 else acc
                acc = np.zeros(nz, complex)
        out[w] = acc
    out[3] = out[3] - (part[0] + part[1])
    out[4] = out[4] + (part[1] - part[0]) - part[2]
    return out


def run_df(prog, g, j):
    """k_zpass_toep_df: one body, imaginary by the kernel index, parity in the two-sided table."""
    nz = j.shape[1]
    part, out = [None] * 3, [None] * 5
    for w in range(5):
        acc = np.zeros(nz, complex)
        for st in range(0 if w < 3 else 1, 3):
            kind, k, c1, c2, neg = decode(prog[w][st])
            v = j[c1] + ((-1.0 if neg else 1.0) * j[c2] if kind == 1 else 0.0)
            acc = acc + toeplitz(g, k, nz, real_body=False) @ v
            if st == 0:
                part[w] = acc
                acc = np.zeros(nz, complex)
        out[w] = acc
    out[3] = out[3] - (part[0] + part[1])
    out[4] = out[4] + (part[1] - part[0]) - part[2]
    return out


def oracle_column(g, j):
    nz = j.shape[1]
    Z = 2 * nz
    S = []
    for k in range(7):
        hc = np.zeros(Z, complex)
        for d in range(-(nz - 1), nz):
            hc[d % Z] = h_two_sided(g, k, d)
        S.append(np.fft.fft(hc))
    F = [np.fft.fft(np.concatenate([j[c], np.zeros(Z - nz)])) for c in range(5)]
    J = solver._tensor_products(S, F)
    return [np.fft.ifft(x)[:nz] for x in J]


def test_program_covers_the_thirteen_convolutions():
    prog = program()
    steps = [decode(c) for w, row in enumerate(prog) for st, c in enumerate(row) if w < 3 or st > 0]
    assert len(steps) == 13
    # imaginary kernels only in the partial steps of warps 0-1 and the combined-input steps
    for w in range(5):
        for st in range(0 if w < 3 else 1, 3):
            kind, k, *_ = decode(prog[w][st])
            if k in IMAG:
                assert kind == 1 or (st == 0 and w < 2), (w, st)
            if kind == 1:
                assert k in IMAG


@pytest.mark.parametrize("nz", [1, 2, 3, 4, 7, 10, 16])
def test_program_matches_the_oracle_product(nz):
    prog = program()
    rng = np.random.default_rng(100 + nz)
    g = kernels(rng, nz)
    j = rng.standard_normal((5, nz)) + 1j * rng.standard_normal((5, nz))
    ref = oracle_column(g, j)
    scale = max(np.abs(r).max() for r in ref)
    for name, got in (("complex64", run_c64(prog, g, j)), ("double-float", run_df(prog, g, j))):
        for c in range(5):
            assert np.abs(got[c] - ref[c]).max() <= 1e-12 * scale, (name, nz, c)


def test_a_wrong_table_is_caught():
    """The check is not vacuous: swapping two steps' kernels changes the product."""
    prog = [row[:] for row in program()]
    rng = np.random.default_rng(7)
    g = kernels(rng, 6)
    j = rng.standard_normal((5, 6)) + 1j * rng.standard_normal((5, 6))
    ref = oracle_column(g, j)
    kind, k, c1, c2, neg = decode(prog[3][1])
    prog[3][1] = kind | 5 << 2 | c1 << 5 | c2 << 8 | neg << 11   # G3 j2 -> G5 j2 in warp 3
    bad = run_c64(prog, g, j)
    assert np.abs(bad[3] - ref[3]).max() > 1e-3 * np.abs(ref[3]).max()
