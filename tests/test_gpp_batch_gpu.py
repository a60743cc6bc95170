"""Batched GPP (sigma_gpp_batch_*) on the GPU: many uneven instances through
one work queue per pass, against the oracle and the single-instance plans.

Bars: FP64 <= 1e-12 relative per output against the oracle and against a
single-instance FP64 plan (same terms, different g-vector splits and
tiles).  Mixed and tensor (FP32-class terms): every achtemp / asxtemp output
within 1e-6 relative when its condition number kappa = sqrt(sum |term|^2) /
|sum| is at most 10, else within max(1e-6 |exact|, 8 * 2^-24 * sqrt(sum
|term|^2)).  The FP32 terms carry independent relative errors of about 1.45
* 2^-24 rms (the roundings of the operands to FP32, which no compensated
summation removes), so an output's error is about 1.45 * 2^-24 * sqrt(sum
|term|^2): 8.6e-8 * kappa relative; the second bound is that model at more
than five standard deviations.  Two outputs of the small set have kappa >
10: instance 0's achtemp[1] (kappa 10.8, within 1e-6 all the same) and
instance 1's achtemp[1] (17 bands, stress fill; kappa 17.2: 1.5e-6 mixed,
1.75e-6 tensor, 2e-7 * kappa).  Graph replays are bit-identical to one
another and to the uncaptured execution.
"""
import numpy as np
import pytest
import torch

import workload as W
from conftest import normwise_err, rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
SINGLE_TOL = 1e-12
MIXED_TOL = 1e-6
FP32_TERM_BOUND = 8 * 2.0 ** -24   # per-term error model of the FP32 path, > 5 sigma

# number_bands, nvband, ncouls, ngpown, seed, stress: ragged on purpose
SMALL = [
    (40, 3, 2048, 100, 31, False),
    (17, 1, 512, 30, 32, True),
    (70, 8, 1300, 130, 33, False),
    (5, 0, 256, 9, 34, False),        # no occupied band: empty second pass
    (128, 2, 4096, 64, 35, True),
    (33, 33, 777, 77, 36, False),     # every band occupied
]


def _dev(a):
    a = np.ascontiguousarray(a)
    if np.iscomplexobj(a):
        a = a.view(np.float64)
    return torch.from_numpy(a.copy()).cuda()


class HostInstance:
    """A host-generated instance copied to the device, with its own outputs."""

    def __init__(self, nb, nv, nc, ng, seed, stress, wx=None, wx_stride=0):
        self.prob = W.gpp_random(nb, nv, nc, ng, seed, stress=stress)
        if wx is not None:
            self.prob = W.GppProblem(**{**self.prob.__dict__, "wx_array": wx})
        self.wx_stride = wx_stride
        p = self.prob
        self.d = [_dev(x) for x in (p.aqsmtemp, p.aqsntemp, p.I_eps_array, p.wtilde_array, p.vcoul)]
        self.wx = _dev(p.wx_array)
        self.ach = torch.zeros(6, dtype=torch.float64, device="cuda")
        self.asx = torch.zeros_like(self.ach)
        self.n1 = torch.zeros(2 * nb, dtype=torch.float64, device="cuda")

    def as_dict(self):
        p = self.prob
        return dict(number_bands=p.number_bands, nvband=p.nvband, ncouls=p.ncouls, ngpown=p.ngpown,
                    inv_igp_index=p.inv_igp_index, indinv=p.indinv, wx_array=self.wx,
                    wx_band_stride=self.wx_stride, occ=p.occ, aqsmtemp=self.d[0], aqsntemp=self.d[1],
                    I_eps_array=self.d[2], wtilde_array=self.d[3], vcoul=self.d[4], achtemp=self.ach,
                    asxtemp=self.asx, acht_n1_loc=self.n1)

    def outputs(self):
        return tuple(t.cpu().numpy().view(np.complex128).copy() for t in (self.ach, self.asx, self.n1))

    def oracle(self):
        return O.gpp(self.prob, wx_band_stride=self.wx_stride)

    def abs2(self):
        return O.gpp_abs2(self.prob, wx_band_stride=self.wx_stride)


def _small_set():
    xs = [HostInstance(*c) for c in SMALL]
    # one instance with per-band frequencies (wx_array[n1][3])
    base = W.gpp_random(23, 2, 600, 40, 37)
    rng = np.random.default_rng(1)
    wxb = np.repeat(base.wx_array[None, :], 23, 0) + rng.uniform(-0.7, 0.7, (23, 1))
    xs.append(HostInstance(23, 2, 600, 40, 37, False, wx=np.ascontiguousarray(wxb).reshape(-1), wx_stride=3))
    return xs


def mixed_bound(exact, abs2):
    """Allowed |error| of each mixed / tensor output: 1e-6 relative for
    every output whose condition number kappa = sqrt(sum |term|^2) / |sum
    term| is at most 10; beyond that the FP32 term-rounding model
    8 * 2^-24 * sqrt(sum |term|^2) (the terms' own FP32 roundings, ~1.5 *
    2^-24 rms, cannot be compensated by the summation)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        kappa = np.sqrt(abs2) / np.abs(exact)
    model = np.maximum(MIXED_TOL * np.abs(exact), FP32_TERM_BOUND * np.sqrt(abs2))
    return np.where(kappa <= 10.0, MIXED_TOL * np.abs(exact), model)


def _check(g, o, prec, abs2=None):
    if prec == 0:
        assert rel_err(g[0], o[0]).max() <= FP64_TOL
        if np.any(o[1] != 0):
            assert rel_err(g[1], o[1]).max() <= FP64_TOL
        else:
            assert np.all(g[1] == 0)
        scale = np.abs(o[2]).max()
        assert np.abs(g[2] - o[2]).max() <= FP64_TOL * 10 * scale
    else:
        a_ach, a_asx = abs2
        assert np.all(np.abs(g[0] - o[0]) <= mixed_bound(o[0], a_ach))
        assert np.all(np.abs(g[1] - o[1]) <= mixed_bound(o[1], a_asx))
        assert normwise_err(g[2], o[2]) <= MIXED_TOL


@pytest.fixture(scope="module")
def small_set(sigma_lib):
    xs = _small_set()
    oracles = [x.oracle() for x in xs]
    abs2 = [x.abs2() for x in xs]
    return xs, oracles, abs2


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_batch_matches_oracle(sigma_lib, small_set, prec):
    xs, oracles, abs2 = small_set
    b = sigma_lib.GppBatch([x.as_dict() for x in xs], precision=prec)
    terms, items, launches = b.info()
    assert terms == sum(x.prob.number_bands * x.prob.ngpown * x.prob.ncouls * 3 for x in xs)
    assert items > 0 and launches >= 2
    b.execute()
    assert b.status() == 0
    b.close()
    for x, o, a in zip(xs, oracles, abs2):
        _check(x.outputs(), o, prec, a)


@pytest.mark.parametrize("tile", [0, 1, 2], ids=["32x32", "16x64", "64x16"])
def test_batch_every_tile_shape_matches_oracle(sigma_lib, small_set, tile):
    xs, oracles, _ = small_set
    b = sigma_lib.GppBatch([x.as_dict() for x in xs], precision=0, tiles=[tile] * len(xs))
    b.execute()
    assert b.status() == 0
    b.close()
    for x, o in zip(xs, oracles):
        _check(x.outputs(), o, 0)


@pytest.mark.parametrize("tile", [3, 4, 5, 6], ids=["y64x32", "y32x64", "y32x32", "y64x16"])
def test_batch_shared_frequency_tiles_match_oracle(sigma_lib, small_set, tile):
    """Instances that all share one frequency set run the shared-factor
    kernel (tiles 3-6); the last band block of each instance runs the
    shortest item of 16-band slabs that holds its bands (1 to 8 slabs over
    the set's 5 to 128 bands)."""
    xs, oracles, _ = small_set
    keep = [k for k, x in enumerate(xs) if x.wx_stride == 0]
    b = sigma_lib.GppBatch([xs[k].as_dict() for k in keep], precision=0, tiles=[tile] * len(keep))
    b.execute()
    assert b.status() == 0
    b.close()
    for k in keep:
        _check(xs[k].outputs(), oracles[k], 0)
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.GppBatch([xs[k].as_dict() for k in keep], precision=0, tiles=[0] * len(keep))
    assert e.value.status == -8


def test_batch_tensor_matches_oracle(sigma_lib, small_set):
    """Tensor form: the shared-frequency instances with enough columns for
    the contraction tiles; same error model as the FP32 path."""
    xs, oracles, abs2 = small_set
    keep = [k for k, x in enumerate(xs) if x.wx_stride == 0 and x.prob.ngpown >= 20]
    b = sigma_lib.GppBatch([xs[k].as_dict() for k in keep], precision=sigma_lib.PREC_TENSOR)
    s = torch.cuda.Stream()
    b.launch_graph(s.cuda_stream)
    s.synchronize()
    assert b.status(s.cuda_stream) == 0
    first = [xs[k].outputs() for k in keep]
    for k, g in zip(keep, first):
        _check(g, oracles[k], 1, abs2[k])
    b.launch_graph(s.cuda_stream)   # replay: bit-identical
    s.synchronize()
    for k, g in zip(keep, first):
        for u, v in zip(xs[k].outputs(), g):
            assert np.array_equal(u, v)
    b.close()
    small = [k for k, x in enumerate(xs) if x.prob.ngpown < 18]
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.GppBatch([xs[k].as_dict() for k in small], precision=sigma_lib.PREC_TENSOR)
    assert e.value.status == -8


def test_batch_mixed_tiles_in_one_queue(sigma_lib, small_set):
    xs, oracles, _ = small_set
    tiles = [k % 3 for k in range(len(xs))]
    b = sigma_lib.GppBatch([x.as_dict() for x in xs], precision=0, tiles=tiles)
    b.execute()
    assert b.status() == 0
    b.close()
    for x, o in zip(xs, oracles):
        _check(x.outputs(), o, 0)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_batch_graph_replay_bitwise(sigma_lib, small_set, prec):
    xs, _, _ = small_set
    b = sigma_lib.GppBatch([x.as_dict() for x in xs], precision=prec)
    b.execute()
    torch.cuda.synchronize()
    ref = [x.outputs() for x in xs]
    s = torch.cuda.Stream()
    for rep in range(3):
        for x in xs:
            for t in (x.ach, x.asx, x.n1):
                t.zero_()
        torch.cuda.synchronize()
        b.launch_graph(s.cuda_stream)
        s.synchronize()
        assert b.status(s.cuda_stream) == 0
        for x, r in zip(xs, ref):
            for u, v in zip(x.outputs(), r):
                assert np.array_equal(u, v)
    with pytest.raises(sigma_lib.SigmaError) as e:
        b.launch_graph(0)  # the legacy default stream cannot be captured
    assert e.value.status == -8
    b.close()


def test_one_shot_batched(sigma_lib, small_set):
    xs, oracles, _ = small_set
    sigma_lib.gpp_batched([x.as_dict() for x in xs], precision=0)
    for x, o in zip(xs, oracles):
        _check(x.outputs(), o, 0)


def test_batch_rejects_bad_instances(sigma_lib):
    x = HostInstance(8, 1, 256, 16, 40, False)
    d = x.as_dict()
    bad = dict(d, inv_igp_index=np.where(np.arange(16) == 3, 257, d["inv_igp_index"]))
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.GppBatch([d, bad])
    assert e.value.status == -2
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.GppBatch([d, dict(d, nvband=9)])
    assert e.value.status == -1
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.GppBatch([d], tiles=[0])    # per-band-kernel tile for shared frequencies
    assert e.value.status == -8
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.GppBatch([d], tiles=[7])    # no such tile
    assert e.value.status == -8
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.GppBatch([d, dict(d, vcoul=None)])
    assert e.value.status == -6


# ------------------------------------------------ the 48-instance production batch
@pytest.fixture(scope="module")
def batch48(sigma_lib):
    import batched
    xs = batched.device_instances()
    yield xs
    del xs
    torch.cuda.empty_cache()


def test_batch48_fp64_equals_single_plans_and_oracle(sigma_lib, batch48):
    xs = batch48
    b = sigma_lib.GppBatch([x.as_dict() for x in xs], precision=0)
    s = torch.cuda.Stream()
    b.launch_graph(s.cuda_stream)
    s.synchronize()
    assert b.status(s.cuda_stream) == 0
    got = [x.outputs() for x in xs]
    for x, g in zip(xs, got):
        r = x.run_single(0)
        assert rel_err(g[0], r[0]).max() <= SINGLE_TOL
        assert rel_err(g[1], r[1]).max() <= SINGLE_TOL
        assert np.abs(g[2] - r[2]).max() <= SINGLE_TOL * 10 * np.abs(r[2]).max()
    # one band of the two smallest instances against the oracle
    for k in sorted(range(len(xs)), key=lambda k: xs[k].ng * xs[k].nc)[:2]:
        prob = xs[k].host_problem()
        for band in (0, xs[k].nb - 1):
            _, _, on1 = O.gpp(prob, band, band + 1)
            assert rel_err(got[k][2][band], on1[band]) <= FP64_TOL
    # a second replay is bit-identical
    b.launch_graph(s.cuda_stream)
    s.synchronize()
    for x, g in zip(xs, got):
        for u, v in zip(x.outputs(), g):
            assert np.array_equal(u, v)
    b.close()


@pytest.mark.parametrize("prec", [1, 2], ids=["mixed", "tensor"])
def test_batch48_within_bar_of_fp64(sigma_lib, batch48, prec):
    xs = batch48
    b64 = sigma_lib.GppBatch([x.as_dict() for x in xs], precision=0)
    b64.execute()
    assert b64.status() == 0
    g64 = [x.outputs() for x in xs]
    b64.close()
    bmx = sigma_lib.GppBatch([x.as_dict() for x in xs], precision=prec)
    bmx.execute()
    assert bmx.status() == 0
    gmx = [x.outputs() for x in xs]
    bmx.close()
    for x, a, m in zip(xs, g64, gmx):
        # sum |term|^2 from a two-band sample (bands are drawn alike), with margin
        s_ach, s_asx = O.gpp_abs2(x.host_problem(), 0, 2)
        k = min(x.nvb, 2)
        ach2 = 1.5 * s_ach * x.nb / 2
        asx2 = 1.5 * s_asx * x.nvb / k
        assert np.all(np.abs(m[0] - a[0]) <= mixed_bound(a[0], ach2))
        assert np.all(np.abs(m[1] - a[1]) <= mixed_bound(a[1], asx2))
        assert normwise_err(m[2], a[2]) <= MIXED_TOL
