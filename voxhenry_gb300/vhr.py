"""The .vhr input format of VoxHenry: reader and writer.

Reader: the keyword-per-line format of src_pre_process/pre_input_file.m:1-133 -- `freq=` lines
(any number of values, repeated lines append), `dx=`, `LMN=L,M,N`, an optional `Superconductor`
keyword, a voxel block between `StartVoxelList` and `EndVoxelList` of `V ix iy iz sigma [lambdaL]`
lines (1-based indices), and `N <port> <P|N|other> ix iy iz <side>` port node lines, where P
marks excitation nodes, N return nodes and any other letter nodes to be grounded.  Tokens split
on blanks, '=' and ','; keywords are case-insensitive; '*' lines are comments.

Writer: the layout of src_pre_process/pre_output_file.m (header comment, ten frequencies per
`freq=` line, `dx`, `LMN`, voxel list, port node lines `N port<k> P|N ix iy iz side`).

Grids are Fortran ordered (x fastest) and indices 1-based, as in the reference.
"""
from __future__ import annotations

import gzip
import re
from dataclasses import dataclass, field

import numpy as np

SIDES = ("-x", "+x", "-y", "+y", "-z", "+z")   # node side names; index + 1 is the panel column
_SPLIT = re.compile(r"[ \f\n\r\t\v=,]+")


@dataclass
class VhrModel:
    sigma_e: np.ndarray                  # (L, M, N) conductivity, Fortran order
    lambdaL: np.ndarray | None           # (L, M, N) London penetration depth, or None
    freq: np.ndarray                     # frequencies as listed
    dx: float
    pnt_lft: list = field(default_factory=list)    # per port: (k, 4) int [ix iy iz side], 1-based
    pnt_rght: list = field(default_factory=list)
    pnt_well_cond: np.ndarray | None = None        # (k, 4) nodes to ground, or None
    portnames: list = field(default_factory=list)

    @property
    def num_ports(self) -> int:
        return len(self.pnt_lft)


def _open_text(path: str) -> str:
    if path.endswith(".gz"):
        with gzip.open(path, "rt") as f:
            return f.read()
    with open(path) as f:
        return f.read()


def read(path: str) -> VhrModel:
    """Reads a .vhr file (plain or gzip)."""
    return parse(_open_text(path))


def parse(text: str) -> VhrModel:
    """Parses the text of a .vhr file (pre_input_file.m:1-133)."""
    freq: list[float] = []
    dx = 1e-6
    shape = None
    supercond = False
    ports: dict[str, tuple[list, list]] = {}
    order: list[str] = []
    ground: list = []
    vox_lines: list[str] = []
    lines = text.splitlines()
    i = 0
    while i < len(lines):
        toks = [t for t in _SPLIT.split(lines[i].strip()) if t]
        i += 1
        if not toks:
            continue
        key = toks[0].lower()
        if key == "freq":
            freq.extend(float(t) for t in toks[1:])
        elif key == "dx" and len(toks) >= 2:
            dx = float(toks[1])
        elif key == "lmn" and len(toks) >= 4:
            shape = (int(toks[1]), int(toks[2]), int(toks[3]))
        elif key == "superconductor":
            supercond = True
        elif key == "startvoxellist":
            while i < len(lines):   # the voxel block: V lines until the first other line
                s = lines[i].strip()
                if not s.startswith(("V", "v")):
                    break
                vox_lines.append(s[1:])
                i += 1
        elif key == "n" and len(toks) >= 7:
            name = toks[1]
            key_n = name.lower()
            if key_n not in ports:
                ports[key_n] = ([], [])
                order.append(name)
            node = [int(toks[3]), int(toks[4]), int(toks[5]), SIDES.index(toks[6]) + 1]
            kind = toks[2].upper()
            if kind == "P":
                ports[key_n][0].append(node)
            elif kind == "N":
                ports[key_n][1].append(node)
            else:
                ground.append(node)
    if shape is None:
        raise ValueError("the file has no LMN line")
    sigma = np.zeros(shape, order="F")
    lam = np.zeros(shape, order="F") if supercond else None
    if vox_lines:
        ncol = 5 if supercond else 4
        vals = np.array(" ".join(vox_lines).split(), dtype=np.float64).reshape(-1, ncol)
        ix = vals[:, :3].astype(np.int64) - 1
        sigma[ix[:, 0], ix[:, 1], ix[:, 2]] = vals[:, 3]
        if supercond:
            lam[ix[:, 0], ix[:, 1], ix[:, 2]] = vals[:, 4]
    lft = [np.array(ports[n.lower()][0], dtype=np.int64).reshape(-1, 4) for n in order]
    rgt = [np.array(ports[n.lower()][1], dtype=np.int64).reshape(-1, 4) for n in order]
    return VhrModel(sigma, lam, np.array(freq if freq else [1.0]), dx, lft, rgt,
                    np.array(ground, dtype=np.int64).reshape(-1, 4) if ground else None, order)


def format_text(m: VhrModel, title: str = "VoxHenry structure") -> str:
    """The .vhr text of a model in pre_output_file.m's layout."""
    out = ["* VoxHenry input file", f"* {title}", "", "* Frequency points (Hz)"]
    fs = [f"{f:g}" for f in np.asarray(m.freq).ravel()]
    for k in range(0, len(fs), 10):
        out.append("freq= " + " ".join(fs[k:k + 10]))
    out += ["", "* Voxel size (m)", f"dx={m.dx:g}", "",
            "* Voxel grid dimension in voxel units; x, y, z", "LMN=%d,%d,%d" % m.sigma_e.shape, ""]
    sc = m.lambdaL is not None
    if sc:
        out += ["* Specify there are superconductors", "Superconductor", ""]
    out += ["* Voxel list", "* Format is:", "* V <index_x> <index_y> <index_z> <conductivity S/m>", "*",
            "StartVoxelList"]
    sig = np.asarray(m.sigma_e)
    occ = (sig != 0) if not sc else ((sig != 0) | (np.asarray(m.lambdaL) != 0))
    lin = np.flatnonzero(occ.ravel(order="F"))
    ix, iy, iz = np.unravel_index(lin, sig.shape, order="F")
    s = sig.ravel(order="F")[lin]
    if sc:
        lmb = np.asarray(m.lambdaL).ravel(order="F")[lin]
        out += [f"V {a + 1} {b + 1} {c + 1} {v:g} {l:g}" for a, b, c, v, l in zip(ix, iy, iz, s, lmb)]
    else:
        out += [f"V {a + 1} {b + 1} {c + 1} {v:g}" for a, b, c, v in zip(ix, iy, iz, s)]
    out += ["EndVoxelList", "", "* Port nodes list", "* Format is:",
            "* N <portname> <excitation or ground (P/N)> <voxel_index_x> <voxel_index_y> <voxel_index_z> "
            "<node (+z,-z,+x,-x,+y,-y)>"]
    names = m.portnames or [f"port{k + 1}" for k in range(m.num_ports)]
    for k in range(m.num_ports):
        out.append("*")
        for tag, nodes in (("P", m.pnt_lft[k]), ("N", m.pnt_rght[k])):
            for a, b, c, sd in np.asarray(nodes).reshape(-1, 4):
                out.append(f"N {names[k]} {tag} {a} {b} {c} {SIDES[sd - 1]}")
    if m.pnt_well_cond is not None and len(m.pnt_well_cond):
        out.append("*")
        for a, b, c, sd in np.asarray(m.pnt_well_cond).reshape(-1, 4):
            out.append(f"N ground G {a} {b} {c} {SIDES[sd - 1]}")
    return "\n".join(out) + "\n"


def write(path: str, m: VhrModel, title: str = "VoxHenry structure") -> None:
    """Writes a .vhr file (gzip when the name ends in .gz)."""
    text = format_text(m, title)
    if path.endswith(".gz"):
        with gzip.open(path, "wt") as f:
            f.write(text)
    else:
        with open(path, "w") as f:
            f.write(text)
