"""The multi-GPU host logic (fortkernels-_gb300/replicas.py) with world
size 2 on CPU (gloo): instance sharding, band ranges, the max-over-ranks
timing reduction and the band-split gather, checked against the oracle run
on the whole instance."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import replicas as R
import workload as W


def test_shard_instances_covers_and_balances():
    terms = [s["number_bands"] * s["ngpown"] * s["ncouls"] * 3 for s in W.batched_shapes()]
    for world in (1, 2, 3, 8):
        parts = R.shard_instances(terms, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(terms)))
        loads = [sum(terms[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(terms)
    assert R.shard_instances([5, 1, 1], 2) == [[0], [1, 2]]


def test_band_ranges_partition():
    for nb in (1, 7, 512):
        for world in (1, 2, 3, 8):
            rs = [R.band_range(nb, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == nb
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            assert max(e - b for b, e in rs) - min(e - b for b, e in rs) <= 1


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # max-over-ranks timing
        out[f"max{rank}"] = R.max_over_ranks(10.0 + rank, dist)
        # band split of one instance: each rank its contiguous bands
        prob = W.gpp_random(9, 3, 256, 12, 71)
        b, e = R.band_range(prob.number_bands, rank, world)
        ach, asx, n1 = O.gpp(prob, b, e, nthreads=1)
        # per-band rows of this rank: the oracle's acht_n1_loc holds [iw=2];
        # the other frequencies come from per-band oracle runs
        rows = np.zeros((e - b, 3), np.complex128)
        for k, band in enumerate(range(b, e)):
            a_b, _, _ = O.gpp(prob, band, band + 1, nthreads=1)
            rows[k] = a_b
        got = R.gather_bands(rows, b, prob.number_bands, asx, dist)
        if rank == 0:
            out["gather"] = got
    finally:
        dist.destroy_process_group()


def test_two_rank_gather_equals_single_instance():
    from oracle import oracle as O
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out["max0"] == out["max1"] == 11.0
        ach, asx, n1 = out["gather"]
    prob = W.gpp_random(9, 3, 256, 12, 71)
    oach, oasx, on1 = O.gpp(prob, nthreads=1)
    assert np.abs(ach - oach).max() <= 1e-13 * np.abs(oach).max()
    assert np.abs(asx - oasx).max() <= 1e-13 * np.abs(oasx).max()
    assert np.abs(n1 - on1).max() <= 1e-13 * np.abs(on1).max()


def test_aggregate_rate():
    assert R.aggregate_rate(100.0, 4, 1000.0) == 400.0
    assert np.isnan(R.aggregate_rate(1.0, 2, 0.0))
