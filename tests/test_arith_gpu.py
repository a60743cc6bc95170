"""Device arithmetic the FP64 path's accuracy claim rests on.

rcp_f64_seed32 forms 1/|wdiff|^2 for every kept term of the FP64 kernels
(the reference divides: BGW-Kernels/gppKer.cpp:397-398): an FP32 seed of the
leading 23 mantissa bits, the exponent rebuilt on the integer pipe, one FP64
Newton step; stated within 2^-44.8 relative for normal w whose reciprocal is
normal.  rcp_f64 (hardware FP64 seed, cubic step) is stated within the FP64
rounding unit.  Both are checked against the correctly rounded IEEE 1/w.
"""
import numpy as np
import pytest
import torch

import workload as W
from conftest import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SEED32_BOUND = 2.0 ** -44.8
RCP64_BOUND = 2.0 ** -52


def _sample_w(n, seed):
    """Normal doubles over exponents -1000..1000 (reciprocals normal), random
    mantissas, plus the edges of the seed: mantissas 1.0 and all ones, the
    23-bit truncation boundary, and the pole-guard range [0.25, 1e7]."""
    rng = np.random.default_rng(seed)
    mant = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    ex = rng.integers(1023 - 1000, 1023 + 1000, n, dtype=np.uint64)
    w = (ex << np.uint64(52) | mant).view(np.float64)
    edges = []
    for e in (-1000, -300, -1, 0, 1, 2, 300, 1000):
        for m in (0, (1 << 52) - 1, (1 << 29) - 1, 1 << 29, ((1 << 23) - 1) << 29, (((1 << 23) - 1) << 29) | 1):
            edges.append(((e + 1023) << 52) | m)
    edges = np.array(edges, dtype=np.uint64).view(np.float64)
    guard = np.exp(rng.uniform(np.log(0.25), np.log(1e7), n // 4))
    return np.concatenate([w, edges, guard])


def test_fp64_reciprocals_within_stated_bounds(sigma_lib):
    w = _sample_w(1 << 20, 5)
    dw = torch.from_numpy(w).cuda()
    out = torch.empty(3 * len(w), dtype=torch.float64, device="cuda")
    st = sigma_lib.load().sigma_eval_reciprocals(dw.data_ptr(), out.data_ptr(), len(w), None)
    assert st == 0
    torch.cuda.synchronize()
    o = out.cpu().numpy().reshape(-1, 3)
    exact = o[:, 2]
    assert np.array_equal(exact, 1.0 / w)  # the device's IEEE 1/w is numpy's
    e_seed = (o[:, 1] - exact) / exact
    e_rcp = (o[:, 0] - exact) / exact
    assert np.abs(e_seed).max() <= SEED32_BOUND, np.abs(e_seed).max()
    assert np.abs(e_rcp).max() <= RCP64_BOUND, np.abs(e_rcp).max()
    # the Newton step approaches 1/w from below (up to the final rounding)
    assert np.all(e_seed <= 2.0 ** -53)


def test_overflowing_wdiff_drops_the_term(sigma_lib):
    """A frequency so large that |wdiff|^2 overflows: the reference's rden is
    1/inf = 0, so every term of that frequency is 0; the FP64 path drops
    them (no garbage reciprocal of inf)."""
    prob = W.gpp_random(20, 0, 1024, 40, 43)
    prob.wx_array = np.array([3.0, 4.0, 1e200])
    ach, asx, _ = O.gpp(prob)
    assert ach[2] == 0 and np.all(asx == 0)
    g = sigma_lib.gpp_host(prob, sigma_lib.PREC_FP64)
    assert g[0][2] == 0
    assert rel_err(g[0][:2], ach[:2]).max() <= 1e-12


def _sample_split(n, seed):
    """Doubles over the split's range and beyond, random mantissas, plus
    remainders of exactly half an FP32 ulp of lo (ties), either side of a
    tie, all-ones mantissas, the range edges, zeros, infinities, NaN."""
    rng = np.random.default_rng(seed)
    sign = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    mant = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    ex = rng.integers(1023 - 160, 1023 + 160, n, dtype=np.uint64)
    x = (sign | ex << np.uint64(52) | mant).view(np.float64)
    special = []
    for e in (-126, -100, -75, -74, -73, -1, 0, 1, 20, 127):
        for m in (1 << 4, (1 << 4) | (1 << 5), (1 << 4) - 1, (1 << 4) + 1, (1 << 52) - 1, (1 << 29) - 1,
                  1 << 29, 0):
            for s in (0, 1):
                special.append((s << 63) | ((e + 1023) << 52) | m)
    sp = np.array(special, dtype=np.uint64).view(np.float64)
    edge = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 3.4028235677973366e38, 1e-40, -1e-45])
    return np.concatenate([x, sp, edge])


def test_float_float_split(sigma_lib):
    """The float-float split behind the FP32-class forms and the FP64 forms'
    float-float factors: hi = x truncated to 24 significant bits and lo =
    the remaining 29 bits rounded to FP32 (so |x - hi - lo| <= 2^-48 |x|)
    over 2^-74 <= |x| < 2^128; below it a signed zero or hi alone, above it
    an infinite hi."""
    x = _sample_split(1 << 20, 7)
    dx = torch.from_numpy(x).cuda()
    out = torch.empty(2 * len(x), dtype=torch.float32, device="cuda")
    assert sigma_lib.load().sigma_eval_split(dx.data_ptr(), out.data_ptr(), len(x), None) == 0
    torch.cuda.synchronize()
    o = out.cpu().numpy().reshape(-1, 2)
    nan = np.isnan(x)
    ax = np.abs(x)
    inside = ~nan & (ax >= 2.0 ** -74) & (ax < 2.0 ** 128)
    xs = x[inside]
    hi = ((xs.view(np.uint64) >> np.uint64(29)) << np.uint64(29)).view(np.float64)  # truncated to 24 bits
    assert np.array_equal(o[inside, 0].astype(np.float64), hi)
    lo = (xs - hi).astype(np.float32)  # x - hi is exact in FP64; one rounding to FP32
    assert np.array_equal(o[inside, 1], lo)  # (a zero lo carries x's sign)
    err = np.abs(xs - o[inside, 0].astype(np.float64) - o[inside, 1].astype(np.float64))
    assert np.all(err <= 2.0 ** -48 * np.abs(xs))
    big = ~nan & (ax >= 2.0 ** 128)
    assert np.all(np.isinf(o[big, 0])) and np.all(o[big, 1] == 0)
    assert np.all(np.isnan(o[nan, 0]))
    tiny = ~nan & (ax < 2.0 ** -126)
    assert np.all(o[tiny, 0] == 0) and np.all(o[tiny, 1] == 0)


def test_float_float_split_round(sigma_lib):
    """The rounded split of the FP64 forms' float-float terms: hi = x rounded
    to the nearest FP32 value (ties to even, numpy's conversion) and lo = x -
    hi rounded to FP32 over 2^-74 <= |x| < 2^128 (hi infinite from FLT_MAX +
    1/2 ulp up); below 2^-74 as the truncated split."""
    x = _sample_split(1 << 20, 8)
    rng = np.random.default_rng(9)
    # ties of hi: the dropped 29 bits exactly half an ulp, kept mantissa odd and even
    ties = []
    for e in (-74, -20, -1, 0, 1, 20, 127):
        for k in rng.integers(0, 1 << 23, 8):
            m = (int(k) << 29) | (1 << 28)
            for s in (0, 1):
                ties.append((s << 63) | ((e + 1023) << 52) | m)
    x = np.concatenate([x, np.array(ties, dtype=np.uint64).view(np.float64)])
    dx = torch.from_numpy(x).cuda()
    out = torch.empty(2 * len(x), dtype=torch.float32, device="cuda")
    assert sigma_lib.load().sigma_eval_split_round(dx.data_ptr(), out.data_ptr(), len(x), None) == 0
    torch.cuda.synchronize()
    o = out.cpu().numpy().reshape(-1, 2)
    nan = np.isnan(x)
    ax = np.abs(x)
    inside = ~nan & (ax >= 2.0 ** -74) & (ax < 2.0 ** 128)
    xs = x[inside]
    with np.errstate(over="ignore"):
        hi = xs.astype(np.float32)
    assert np.array_equal(o[inside, 0], hi)
    fin = np.isfinite(hi)
    lo = (xs[fin] - hi[fin].astype(np.float64)).astype(np.float32)  # exact in FP64, one rounding
    assert np.array_equal(o[inside, 1][fin], lo)
    err = np.abs(xs[fin] - hi[fin].astype(np.float64) - lo.astype(np.float64))
    assert np.all(err <= 2.0 ** -48 * np.abs(xs[fin]))
    assert np.all(np.abs(lo.astype(np.float64)) <= 2.0 ** -24 * np.abs(xs[fin]))
    big = ~nan & (ax >= 2.0 ** 128)
    assert np.all(np.isinf(o[big, 0])) and np.all(o[big, 1] == 0)
    assert np.all(np.isnan(o[nan, 0]))
    tiny = ~nan & (ax < 2.0 ** -126)
    assert np.all(o[tiny, 0] == 0) and np.all(o[tiny, 1] == 0)
