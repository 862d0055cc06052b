"""Oracle: .vhr input reader and structure parameters (test infrastructure).

Restates src_pre_process/pre_input_file.m:1-133 and
src_pre_process/pre_define_structure_params.m:1-26 of the reference.
Arrays follow the reference's MATLAB conventions: 3-D grids are Fortran
ordered (x fastest) and voxel/port indices are 1-based.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np

# pre_input_file.m:9 -- node side names, index+1 is the column of all_panels_ids
SIDES = ("-x", "+x", "-y", "+y", "-z", "+z")


@dataclass
class VhrInput:
    sigma_e: np.ndarray            # (L, M, N) float64, Fortran order
    lambdaL: np.ndarray | None     # (L, M, N) or None for normal conductors
    freq: np.ndarray               # (nfreq,) float64, as read (unsorted)
    dx: float
    pnt_lft: list = field(default_factory=list)   # per port: (k, 4) int [x y z side] 1-based
    pnt_rght: list = field(default_factory=list)
    pnt_well_cond: np.ndarray | None = None        # (k, 4) or None

    @property
    def num_ports(self) -> int:
        return len(self.pnt_lft)


def read_vhr_text(text: str) -> VhrInput:
    """pre_input_file.m:35-133: tokenise each line on blanks, '=' and ','."""
    freq: list[float] = []
    dx = 1e-6                       # pre_input_file.m:21
    sigma_e = None
    lambdaL = None
    supercond = False
    portnames: list[str] = []
    pnt_lft: list[list] = []
    pnt_rght: list[list] = []
    well: list = []
    lines = text.splitlines()
    i = 0
    while i < len(lines):
        toks = [t for t in re.split(r"[ \f\n\r\t\v=,]+", lines[i].strip()) if t != ""]
        i += 1
        if not toks:
            continue
        key = toks[0].lower()
        if key == "freq":
            freq.extend(float(t) for t in toks[1:])
        elif key == "dx":
            if len(toks) >= 2:
                dx = float(toks[1])
        elif key == "lmn":
            if len(toks) >= 4:
                L, M, N = (int(float(t)) for t in toks[1:4])
                sigma_e = np.zeros((L, M, N), order="F")
                lambdaL = np.zeros((L, M, N), order="F")
        elif key == "superconductor":
            supercond = True
        elif key == "startvoxellist":
            # textscan('V %d %d %d %f [%f]') until the first non-matching line
            while i < len(lines):
                vt = lines[i].split()
                if len(vt) < (6 if supercond else 5) or vt[0] != "V":
                    break
                x, y, z = int(vt[1]) - 1, int(vt[2]) - 1, int(vt[3]) - 1
                sigma_e[x, y, z] = float(vt[4])
                if supercond:
                    lambdaL[x, y, z] = float(vt[5])
                i += 1
        elif key == "n":
            if len(toks) >= 7:
                pname = toks[1]
                low = [p.lower() for p in portnames]
                if pname.lower() in low:
                    pnum = low.index(pname.lower())
                else:
                    portnames.append(pname)
                    pnt_lft.append([])
                    pnt_rght.append([])
                    pnum = len(portnames) - 1
                row = [int(toks[3]), int(toks[4]), int(toks[5]), SIDES.index(toks[6]) + 1]
                kind = toks[2].lower()
                if kind == "p":
                    pnt_lft[pnum].append(row)
                elif kind == "n":
                    pnt_rght[pnum].append(row)
                else:
                    well.append(row)
    if not supercond:
        lambdaL = None              # pre_input_file.m:112-114
    return VhrInput(
        sigma_e=sigma_e,
        lambdaL=lambdaL,
        freq=np.asarray(freq if freq else [1.0], dtype=np.float64),
        dx=dx,
        pnt_lft=[np.asarray(p, dtype=np.int64).reshape(-1, 4) for p in pnt_lft],
        pnt_rght=[np.asarray(p, dtype=np.int64).reshape(-1, 4) for p in pnt_rght],
        pnt_well_cond=np.asarray(well, dtype=np.int64).reshape(-1, 4) if well else None,
    )


def read_vhr(path: str) -> VhrInput:
    with open(path, "r") as f:
        return read_vhr_text(f.read())


def structure_params(sigma_e: np.ndarray, lambdaL: np.ndarray | None):
    """pre_define_structure_params.m:1-16 -> (idxS, idxS5), 1-based linear indices."""
    L, M, N = sigma_e.shape
    nD = L * M * N
    nz = np.abs(sigma_e.ravel(order="F")) > 1e-12
    if lambdaL is not None:
        nz = nz | (np.abs(lambdaL.ravel(order="F")) > 1e-12)
    idxS = np.flatnonzero(nz).astype(np.int64) + 1
    idxS5 = np.concatenate([idxS + k * nD for k in range(5)])
    return idxS, idxS5
