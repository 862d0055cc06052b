"""Frequency sharding of a sweep over the ranks of a torch.distributed group.

Every (frequency, port) solve of VoxHenry_executer.m:215-329 is independent, and a frequency's
ports share its Schur factor, so a sweep splits by frequency: each rank keeps its own geometry
(tensor, Ae, factors) on its own GPU and solves a disjoint subset of the frequencies.  The only
communication is the gather of the small per-frequency results (R, L, flags) at the end; nothing
is exchanged on the data path.
"""
from __future__ import annotations

from typing import Callable

import numpy as np


def shard_frequencies(nfreq: int, rank: int, world: int) -> np.ndarray:
    """Indices of the frequencies rank `rank` solves: round robin, so that every rank gets a share of
    the slow high-frequency points (GMRES iterations grow with frequency)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    return np.arange(rank, nfreq, world, dtype=np.int64)


def gather_sweep(local: dict, idx: np.ndarray, nfreq: int, group=None) -> dict:
    """All-gathers the per-frequency results {"R", "L", "flag"} of every rank's shard (leading axis
    = the rank's frequencies, in `idx` order) into full arrays on every rank."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (np.asarray(idx), {k: np.asarray(v) for k, v in local.items()}), group=group)
    out = {}
    for k in local:
        sample = np.asarray(local[k])
        full = np.zeros((nfreq,) + sample.shape[1:], dtype=sample.dtype)
        for pidx, pres in parts:
            full[pidx] = pres[k]
        out[k] = full
    return out


def sweep_distributed(freqs, solve: Callable[[np.ndarray], dict], group=None) -> dict:
    """Solves this rank's share of `freqs` with `solve(freqs_subset) -> {"R", "L", "flag", ...}` and
    returns the full sweep on every rank (only the keys R, L and flag are gathered)."""
    import torch.distributed as dist

    freqs = np.asarray(freqs, dtype=np.float64)
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    idx = shard_frequencies(len(freqs), rank, world)
    res = solve(freqs[idx]) if len(idx) else None
    if res is None:   # a rank without frequencies still takes part in the gather
        P = solve.num_ports if hasattr(solve, "num_ports") else 1
        res = {"R": np.zeros((0, P, P)), "L": np.zeros((0, P, P)), "flag": np.zeros((0,), dtype=np.int32)}
    local = {"R": res["R"], "L": res["L"], "flag": np.asarray(res["flag"]).reshape(len(idx), -1).max(axis=1)}
    return gather_sweep(local, idx, len(freqs), group)


def gpu_sweep_solver(prob, tol=None, restart=50, maxit=10, prec="fp64", precon="schur_invert"):
    """The `solve` callable of sweep_distributed for this rank's GPU: a Sweep over the given frequencies."""
    from . import executer

    def solve(fs):
        sw = executer.Sweep(prob, fs, precon=precon).prepare()
        out = sw.solve(restart=restart, tol=tol, maxit=maxit, prec=prec)
        return {"R": out["R"], "L": out["L"], "flag": out["flag"]}

    solve.num_ports = prob.num_ports
    return solve
