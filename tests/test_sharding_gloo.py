"""Frequency sharding over 2 gloo ranks on CPU: the gathered R, L equal a one-process sweep.

The per-rank solve is the oracle's (test infrastructure; the GPU solver plugs into the same
sweep_distributed call through sharding.gpu_sweep_solver)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from oracle import circulant, solver
from oracle import structure as ostruct
from voxhenry_gb300 import geometry, sharding


def _problem():
    w = geometry.two_bars(L=16, M=10, N=5, xr=(1, 15), zr=(1, 3), y1=(1, 3), y2=(6, 8))
    S = ostruct.build_system(w.sigma_e, None, w.dx, w.pnt_lft, w.pnt_rght)
    fN, st = circulant.generate_circulant_tensor(w.dx, 1.0, S.L, S.M, S.N)
    return S, fN, st


FREQS = np.array([1e3, 1e6, 1e8, 1e9, 5e9])


def _oracle_solver(S, fN, st):
    def solve(fs):
        out = solver.solve_frequencies(S, fN, st, np.asarray(fs), restart=50, tol=1e-10)
        return {"R": out["R"], "L": out["L"], "flag": np.zeros(len(fs), dtype=np.int32)}

    solve.num_ports = S.rhs.shape[1]
    return solve


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        S, fN, st = _problem()
        out = sharding.sweep_distributed(FREQS, _oracle_solver(S, fN, st))
        q.put((rank, out["R"], out["L"], sharding.shard_frequencies(len(FREQS), rank, world)))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shards_are_disjoint_and_complete():
    for n, world in [(32, 1), (32, 3), (5, 8), (7, 2)]:
        parts = [sharding.shard_frequencies(n, r, world) for r in range(world)]
        allidx = np.concatenate(parts)
        assert sorted(allidx.tolist()) == list(range(n))


def test_two_gloo_ranks_gather_the_full_sweep():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    S, fN, st = _problem()
    ref = solver.solve_frequencies(S, fN, st, FREQS, restart=50, tol=1e-10)
    for rank, R, L, idx in res:
        assert len(idx) in (2, 3)
        np.testing.assert_allclose(R, ref["R"], rtol=1e-12)   # every rank holds the whole sweep
        np.testing.assert_allclose(L, ref["L"], rtol=1e-12)
