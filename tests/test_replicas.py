"""Replica partitioning and the N > 1 host path, run as world-size-2 gloo
process groups on CPU (the per-rank solver is the oracle here; the GPU run
uses the same functions with NCCL)."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

from ligmg_gb300.replicas import block_range, lpt_partition


def test_block_range_covers_everything():
    for total in (0, 1, 7, 32, 33):
        for world in (1, 2, 3, 8):
            ranges = [block_range(total, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == total
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c and a <= b
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1


def test_lpt_partition_balances():
    w = np.random.default_rng(0).lognormal(0, 1, 256)
    parts = lpt_partition(w, 4)
    assert sorted(sum(parts, [])) == list(range(256))
    loads = [w[p].sum() for p in parts]
    assert max(loads) <= min(loads) + w.max()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


NGRAPHS, NBLOCKS = 5, 6


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from ligmg_gb300 import graphs as G
    from ligmg_gb300.replicas import lpt_partition, reduce_max, reduce_sum
    from oracle import oracle as O
    O.set_threads(1)
    gs = [G.grid2d(12 + 3 * i, weights="lognormal", seed=i) for i in range(NGRAPHS)]
    # graphs are the unit split across ranks; every rank solves all RHS
    # blocks of the graphs it owns
    mine = lpt_partition([g.nnz for g in gs], world)[rank]
    res = {}
    for gi in mine:
        S = O.OracleSolver(gs[gi], kcycle=1, outer_ksp_type="fcg")
        for c in range(NBLOCKS):
            x, info = S.solve(G.rhs(gs[gi].n, seed=100 * gi + c))
            res[(gi, c)] = (info["iters"], float(info["true_rel_residual"]))
    tmax = reduce_max([float(rank + 1)])
    cnt = reduce_sum([float(len(res))])
    out[rank] = (res, tmax[0], cnt[0])
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    world, port = 2, _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    allres = {}
    for r in range(world):
        res, tmax, cnt = out[r]
        assert tmax == 2.0  # max over ranks
        assert not (set(res) & set(allres))  # no pair solved by two ranks
        allres.update(res)
    # every (graph, rhs-block) pair was solved, by exactly one rank
    assert set(allres) == {(g, c) for g in range(NGRAPHS) for c in range(NBLOCKS)}
    assert out[0][2] == out[1][2] == float(NGRAPHS * NBLOCKS)
    for (gi, c), (iters, tr) in allres.items():
        assert iters > 0 and tr < 1e-7
    # graphs were split between the two ranks
    g0 = {k[0] for k in out[0][0]}
    g1 = {k[0] for k in out[1][0]}
    assert g0 and g1 and not (g0 & g1)
