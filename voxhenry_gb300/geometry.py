"""Seeded synthetic voxel geometries for the benchmark and test workloads.

Each builder returns a ``Workload``: the conductivity grid sigma_e (L, M, N) in
the reference's column-major convention, voxel size dx, the port node lists
in the .vhr form of src_pre_process/pre_input_file.m:68-100 (rows
[x y z side], 1-based, side 1..6 = -x,+x,-y,+y,-z,+z), and the frequencies.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SEED = 20261203
SIDE = {"-x": 1, "+x": 2, "-y": 3, "+y": 4, "-z": 5, "+z": 6}


@dataclass
class Workload:
    name: str
    sigma_e: np.ndarray
    dx: float
    pnt_lft: list
    pnt_rght: list
    freqs: np.ndarray
    lambdaL: np.ndarray | None = None
    tol: float = 1e-8
    restart: int = 50
    maxit: int = 10
    meta: dict = field(default_factory=dict)

    @property
    def shape(self):
        return self.sigma_e.shape


def face_nodes(mask: np.ndarray, side: str) -> np.ndarray:
    """Port node rows [x y z side] (1-based) for every voxel of `mask`."""
    idx = np.argwhere(mask)
    return np.concatenate([idx + 1, np.full((idx.shape[0], 1), SIDE[side])], axis=1).astype(np.int64)


def bar(L=64, M=16, N=16, dx=0.5e-6, sigma=5.8e7, freqs=None) -> Workload:
    """Single straight bar filling the grid; port from the x=1 faces to the x=L faces."""
    s = np.full((L, M, N), sigma, order="F")
    occ = s > 0
    lft = face_nodes(np.pad(occ[:1], ((0, L - 1), (0, 0), (0, 0))), "-x")
    rgt = face_nodes(np.pad(occ[-1:], ((L - 1, 0), (0, 0), (0, 0))), "+x")
    f = np.logspace(3, 10, 8) if freqs is None else np.asarray(freqs, dtype=np.float64)
    return Workload("bar", s, dx, [lft], [rgt], f, tol=1e-8, restart=50)


def two_bars(L=128, M=64, N=32, dx=1e-6, freqs=None, xr=(14, 114), zr=(11, 21), y1=(12, 22), y2=(42, 52),
             sigmas=(5.8e7, 3.5e7)) -> Workload:
    """Copper (5.8e7) and aluminium (3.5e7) bars 100 x 10 x 10 voxels, 20-voxel gap, one port each
    (0-based half-open voxel ranges)."""
    s = np.zeros((L, M, N), order="F")
    xs, zs = slice(*xr), slice(*zr)
    s[xs, slice(*y1), zs] = sigmas[0]
    s[xs, slice(*y2), zs] = sigmas[1]
    lft, rgt = [], []
    for ys in (slice(*y1), slice(*y2)):
        m1 = np.zeros(s.shape, bool)
        m1[xr[0], ys, zs] = True
        m2 = np.zeros(s.shape, bool)
        m2[xr[1] - 1, ys, zs] = True
        lft.append(face_nodes(m1, "-x"))
        rgt.append(face_nodes(m2, "+x"))
    f = np.logspace(3, 10, 16) if freqs is None else np.asarray(freqs, dtype=np.float64)
    return Workload("two_bars", s, dx, lft, rgt, f)


def square_spiral(L=256, M=256, N=8, dx=1e-6, turns=4, width=5, thick=4, space=2, inset=2, sigma=5.8e7,
                  freqs=None) -> Workload:
    """Rectangular spiral coil winding inwards; port between the outer and the inner trace end."""
    s = np.zeros((L, M, N), order="F")
    pitch = width + space
    zs = slice(0, thick)
    lo_prev = inset
    last = None
    for t in range(turns):
        lo = inset + pitch * t
        hix = L - 1 - inset - pitch * t
        hiy = M - 1 - inset - pitch * t
        if hix - lo < 2 * width + space or hiy - lo < 2 * width + space:
            break
        x0 = inset if t == 0 else lo_prev
        s[x0:hix + 1, lo:lo + width, zs] = sigma                 # bottom, +x
        s[hix - width + 1:hix + 1, lo:hiy + 1, zs] = sigma         # right, +y
        s[lo:hix + 1, hiy - width + 1:hiy + 1, zs] = sigma         # top, -x
        s[lo:lo + width, lo + pitch:hiy + 1, zs] = sigma           # left, -y (stops one pitch short)
        last = lo
        lo_prev = lo
    m1 = np.zeros(s.shape, bool)
    m1[inset, inset:inset + width, zs] = True
    m2 = np.zeros(s.shape, bool)
    m2[last:last + width, last + pitch, zs] = True
    f = np.logspace(6, np.log10(2e10), 32) if freqs is None else np.asarray(freqs, dtype=np.float64)
    return Workload("square_spiral", s, dx, [face_nodes(m1, "-x")], [face_nodes(m2, "-y")], f,
                    meta={"turns": turns})


def ring(L=512, M=512, N=16, dx=1e-6, radius=150.0, width=10, z0=3, gap=2, sigma=5.8e7, freqs=None) -> Workload:
    """Single-turn ring (square cross-section, centre-in-ring voxelisation) cut by a gap on +x."""
    s = np.zeros((L, M, N), order="F")
    cx, cy = (L + 1) / 2.0, (M + 1) / 2.0
    i = np.arange(1, L + 1)[:, None]
    j = np.arange(1, M + 1)[None, :]
    r = np.sqrt((i - cx) ** 2 + (j - cy) ** 2)
    disk = (r >= radius - width / 2) & (r <= radius + width / 2)
    jg = int(np.floor(cy)) - gap // 2 + 1          # first gap row (1-based)
    gap_rows = np.arange(jg, jg + gap)
    cut = (i > cx) & np.isin(j, gap_rows)
    ring2d = disk & ~cut
    s[:, :, z0:z0 + width] = np.where(ring2d[:, :, None], sigma, 0.0)
    below, above = jg - 1, jg + gap                  # 1-based rows next to the gap
    m1 = np.zeros(s.shape, bool)
    m1[:, below - 1, z0:z0 + width] = (ring2d[:, below - 1] & (np.arange(1, L + 1) > cx))[:, None]
    m2 = np.zeros(s.shape, bool)
    m2[:, above - 1, z0:z0 + width] = (ring2d[:, above - 1] & (np.arange(1, L + 1) > cx))[:, None]
    f = np.logspace(6, np.log10(2e10), 16) if freqs is None else np.asarray(freqs, dtype=np.float64)
    return Workload("ring", s, dx, [face_nodes(m1, "+y")], [face_nodes(m2, "-y")], f)


def cylinder(L, M, N, dx, diameter, sigma, freqs) -> Workload:
    """Wire along x with a voxelised circular cross-section (centre-in-disc test)."""
    s = np.zeros((L, M, N), order="F")
    cy, cz = (M + 1) / 2.0, (N + 1) / 2.0
    j = np.arange(1, M + 1)[:, None]
    k = np.arange(1, N + 1)[None, :]
    disc = (j - cy) ** 2 + (k - cz) ** 2 <= (diameter / 2.0) ** 2
    s[:, disc] = sigma
    occ = s > 0
    m1 = np.zeros(s.shape, bool)
    m1[0] = occ[0]
    m2 = np.zeros(s.shape, bool)
    m2[-1] = occ[-1]
    return Workload("cylinder", s, dx, [face_nodes(m1, "-x")], [face_nodes(m2, "+x")], np.asarray(freqs, float))


def random_blob(shape, fill=0.6, seed=SEED, sigma=(3.5e7, 5.8e7), dx=1e-6) -> Workload:
    """Random occupancy with a full slab at x=1 and x=L so that a port exists (test geometries)."""
    rng = np.random.default_rng(seed)
    L, M, N = shape
    occ = rng.random(shape) < fill
    occ[0] = True
    occ[-1] = True
    occ[:, 0, 0] = True      # keep the two ends connected
    s = np.where(occ, rng.uniform(sigma[0], sigma[1], size=shape), 0.0)
    s = np.asfortranarray(s)
    m1 = np.zeros(shape, bool)
    m1[0] = True
    m2 = np.zeros(shape, bool)
    m2[-1] = True
    return Workload("random_blob", s, dx, [face_nodes(m1, "-x")], [face_nodes(m2, "+x")], np.array([1e3, 1e9]))


# the benchmark workloads by name (default arguments give their full sizes)
WORKLOADS = {
    "bar_64x16x16": bar,
    "square_spiral_256x256x8": square_spiral,
    "two_bars_128x64x32": two_bars,
    "ring_512x512x16": ring,
}


def from_vhr(path_or_model, name: str | None = None) -> Workload:
    """A workload from a .vhr file (or a parsed vhr.VhrModel): the inputs of VoxHenry_executer.m."""
    from . import vhr

    m = vhr.read(path_or_model) if isinstance(path_or_model, str) else path_or_model
    lam = m.lambdaL if m.lambdaL is not None and np.any(m.lambdaL) else None
    return Workload(name or (path_or_model if isinstance(path_or_model, str) else "vhr"), m.sigma_e, m.dx,
                    list(m.pnt_lft), list(m.pnt_rght), np.asarray(m.freq, dtype=np.float64), lambdaL=lam,
                    meta={"pnt_well_cond": m.pnt_well_cond, "portnames": m.portnames})
