"""Host logic of the multi-GPU layout: one process per GPU, no collective on
the data path.

The GPP sum shards two ways (the reference's own MPI design splits columns,
BGW-Kernels/gppKer.cpp:175-176; here bands or whole instances):

  * instances: a batch of independent sigma instances (q-points, band
    windows) is split across ranks by `shard_instances`, largest first onto
    the least-loaded rank, so every rank gets about the same number of terms;
  * bands: one instance's bands are split into contiguous ranges
    (`band_range`); each rank evaluates its range and the only exchange is
    the per-band results, summed on rank 0 in band order by `gather_bands`
    (3 + 3 + number_bands complex values, compensated, so the result does
    not depend on the number of ranks' roundings beyond the per-band sums).

`max_over_ranks` is the timing reduction of the benchmark (the slowest rank
defines the step time).  Everything here runs on CPU tensors with the gloo
backend as well as with NCCL.
"""
from __future__ import annotations

import math

import numpy as np


def rank_seed(base: int, rank: int) -> int:
    """Seed of rank `rank`'s independent instance in replica runs."""
    return base + rank


def shard_instances(terms, world: int):
    """Instance indices per rank: largest first onto the least-loaded rank
    (ties to the lower rank), each rank's list in ascending order."""
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in sorted(range(len(terms)), key=lambda k: (-terms[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += terms[i]
    return [sorted(x) for x in out]


def band_range(number_bands: int, rank: int, world: int):
    """Contiguous band range [begin, end) of `rank` (sizes differ by at most one)."""
    base, extra = divmod(number_bands, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, dist=None) -> float:
    """Maximum of `value` over all ranks (the value itself without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _neumaier(values):
    s = 0.0
    c = 0.0
    for x in values:
        t = s + x
        c += (s - t) + x if abs(s) >= abs(x) else (x - t) + s
        s = t
    return s + c


def gather_bands(n1_part, begin: int, number_bands: int, asx_part, dist=None):
    """Band-split reduction.  Each rank passes its bands' complex
    acht_n1[n1][3] rows (`n1_part`, shape [end-begin][3]) and its asxtemp
    partial [3]; rank 0 returns (achtemp[3], asxtemp[3], acht_n1_loc[nb]) as
    complex128, summed in band (and rank) order with compensation; other
    ranks return None."""
    n1_part = np.asarray(n1_part, dtype=np.complex128).reshape(-1, 3)
    asx_part = np.asarray(asx_part, dtype=np.complex128).reshape(3)
    world = 1 if dist is None or not dist.is_initialized() else dist.get_world_size()
    rank = 0 if world == 1 else dist.get_rank()
    full = np.zeros((number_bands, 3), np.complex128)
    asx_parts = [asx_part]
    if world == 1:
        full[begin:begin + len(n1_part)] = n1_part
    else:
        payload = {"begin": begin, "n1": n1_part, "asx": asx_part}
        got = [None] * world
        dist.all_gather_object(got, payload)
        asx_parts = []
        for g in got:  # rank order
            full[g["begin"]:g["begin"] + len(g["n1"])] = g["n1"]
            asx_parts.append(g["asx"])
    if rank != 0:
        return None
    ach = np.array([complex(_neumaier(full[:, k].real), _neumaier(full[:, k].imag)) for k in range(3)])
    asx = np.array([complex(_neumaier([a[k].real for a in asx_parts]), _neumaier([a[k].imag for a in asx_parts]))
                    for k in range(3)])
    return ach, asx, full[:, 2].copy()


def aggregate_rate(units_per_rank: float, world: int, ms_max: float) -> float:
    """Whole-job rate: all ranks' units over the slowest rank's time (per second)."""
    if ms_max <= 0 or not math.isfinite(ms_max):
        return float("nan")
    return units_per_rank * world / (ms_max * 1e-3)
