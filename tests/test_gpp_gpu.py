"""GPP parity on the GPU, through the C ABI, against the CPU oracle.

Bars (written in each test): FP64 path <= 1e-12 relative per output, mixed
path <= 1e-6 relative per achtemp / asxtemp output.  acht_n1_loc is checked
per band for FP64 and normwise for the mixed path.  On the seeded random
cases the mixed and tensor bar is 1e-6 relative for every output whose
condition number kappa = sqrt(sum |term|^2) / |sum| is at most 10, else
max(1e-6 |exact|, 8 * 2^-24 * sqrt(sum |term|^2)): FP32 terms carry
independent errors of ~1.5 * 2^-24 rms, so an output whose terms cancel can
sit above 1e-6 relative while within the method's error; the second bound is
that model at more than five standard deviations.  The largest kappa of
these cases is 10.06 (nb33-nv1-nc1000-ng37, asxtemp[0]: 5.3e-7 mixed).
"""
import numpy as np
import pytest
import torch

import workload as W
from conftest import normwise_err, rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6
FP32_TERM_BOUND = 8 * 2.0 ** -24


def _mixed_bound(exact, abs2):
    """Allowed |error| of each mixed / tensor output: 1e-6 relative for
    every output whose condition number kappa = sqrt(sum |term|^2) / |sum
    term| is at most 10; beyond that the FP32 term-rounding model
    8 * 2^-24 * sqrt(sum |term|^2) (the terms' own FP32 roundings, ~1.5 *
    2^-24 rms, cannot be compensated by the summation)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        kappa = np.sqrt(abs2) / np.abs(exact)
    model = np.maximum(MIXED_TOL * np.abs(exact), FP32_TERM_BOUND * np.sqrt(abs2))
    return np.where(kappa <= 10.0, MIXED_TOL * np.abs(exact), model)


def _check(g, o, prec, check_n1=True, abs2=None):
    ach, asx, n1 = g
    oach, oasx, on1 = o
    if prec == 1 and abs2 is not None:
        assert np.all(np.abs(ach - oach) <= _mixed_bound(oach, abs2[0]))
        assert np.all(np.abs(asx - oasx) <= _mixed_bound(oasx, abs2[1]))
        if check_n1:
            assert normwise_err(n1, on1) <= MIXED_TOL
        return
    if prec == 0:
        assert rel_err(ach, oach).max() <= FP64_TOL
        if np.any(oasx != 0):
            assert rel_err(asx, oasx).max() <= FP64_TOL
        else:
            assert np.all(asx == 0)
        if check_n1:
            scale = np.abs(on1).max()
            assert np.abs(n1 - on1).max() <= FP64_TOL * 10 * scale
            nz = np.abs(on1) > 1e-3 * scale
            assert rel_err(n1[nz], on1[nz]).max() <= 1e-10
    else:
        assert rel_err(ach, oach).max() <= MIXED_TOL
        if np.any(oasx != 0):
            assert rel_err(asx, oasx).max() <= MIXED_TOL
        if check_n1:
            assert normwise_err(n1, on1) <= MIXED_TOL


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("shape", [(16, 2, 1024, 8), (128, 2, 8192, 20)], ids=lambda s: "x".join(map(str, s)))
def test_constant_fill_matches_oracle_and_closed_form(sigma_lib, shape, prec):
    prob = W.gpp_constant(*shape)
    o = O.gpp(prob)
    g = sigma_lib.gpp_host(prob, prec)
    _check(g, o, prec)
    # closed form of the constant fill (BGW-Kernels/gppKer.cpp fill :275-291)
    nb, ng, nc = prob.number_bands, prob.ngpown, prob.ncouls
    wt, wx = 0.5 + 0.5j, W.wx_frequencies()
    exact = nb * ng * nc * 0.25 * (wt * np.conj(wx - wt) / np.abs(wx - wt) ** 2) * (0.5 + 0.5j)
    assert rel_err(g[0], exact).max() <= (FP64_TOL if prec == 0 else MIXED_TOL)


RANDOM_CASES = [
    # number_bands, nvband, ncouls, ngpown, seed, stress
    (40, 3, 2048, 100, 11, False),
    (40, 3, 2048, 100, 12, True),
    (33, 1, 1000, 37, 13, False),       # ragged: nc not a multiple of the chunk, ng not of the tile
    (7, 0, 333, 5, 14, False),          # no occupied band: asxtemp = 0
    (9, 9, 777, 21, 15, True),          # every band occupied
    (1, 1, 64, 1, 16, False),           # smallest
    (70, 8, 4096, 64, 17, False),       # several band blocks and occupied-band items
]


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("case", RANDOM_CASES, ids=lambda c: f"nb{c[0]}-nv{c[1]}-nc{c[2]}-ng{c[3]}{'-stress' if c[5] else ''}")
def test_random_matches_oracle(sigma_lib, case, prec):
    nb, nvb, nc, ng, seed, stress = case
    prob = W.gpp_random(nb, nvb, nc, ng, seed, stress=stress)
    o = O.gpp(prob)
    g = sigma_lib.gpp_host(prob, prec)
    _check(g, o, prec, abs2=O.gpp_abs2(prob) if prec == 1 else None)


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "mixed", "tensor"])
def test_exact_poles_and_skipped_columns(sigma_lib, prec):
    """Exact poles, a term exactly on the |wdiff|^2 = 0.25 boundary, a zero
    wtilde and |wtilde|^2 >= 62000 (the guard's second condition binding):
    in the tensor form these take the factor pass's out-of-line decisions."""
    prob = W.gpp_random(20, 4, 1024, 30, 21)
    prob.wtilde_array = prob.wtilde_array.copy()
    wx = prob.wx_array
    # exact poles (|wdiff| = 0), points on the guard boundary region, a zero wtilde
    prob.wtilde_array[2, 10] = complex(wx[0], 0.0)
    prob.wtilde_array[5, 11] = complex(wx[2], 0.0)
    prob.wtilde_array[7, 12] = complex(wx[1] + 0.5, 0.0)
    prob.wtilde_array[8, 13] = 0.0
    prob.wtilde_array[9, 14] = complex(300.0, 0.5)
    # skipped columns: igp < 0 (gppKer.cpp:328)
    prob.indinv = prob.indinv.copy()
    prob.indinv[prob.inv_igp_index[3]] = -1
    prob.indinv[prob.inv_igp_index[4]] = -7
    o = O.gpp(prob)
    g = sigma_lib.gpp_host(prob, prec)
    for x in g:
        assert np.all(np.isfinite(x))
    _check(g, o, prec)


@pytest.mark.parametrize("per_band", [False, True], ids=["shared-wx", "per-band-wx"])
@pytest.mark.parametrize("kind", ["huge-elements", "tiny-ieps", "tiny-frequency"])
def test_fp64_outside_float_range(sigma_lib, kind, per_band):
    """The FP64 passes form their factors (the per-band pass: its whole
    terms) in float-float (FP32 pairs) when wtilde, I_eps, aqsn and the
    frequency lie within 2^+-20; other elements take their FP64 fallback.
    Elements with |wtilde| ~ 2^45 and |I_eps| ~ 2^40 (FP32 would overflow),
    an I_eps scaled by 2^-110 (the low FP32 halves would fall below the
    normal range) and a frequency of 1e-7 must all stay within the FP64 bar
    of 1e-12, with one frequency set for all bands and with per-band
    frequencies."""
    prob = W.gpp_random(24, 5, 1200, 40, 31)
    prob.wtilde_array = prob.wtilde_array.copy()
    prob.I_eps_array = prob.I_eps_array.copy()
    if kind == "huge-elements":
        prob.wtilde_array[3, 17] *= 2.0 ** 45
        prob.wtilde_array[11, 400:404] *= 2.0 ** 30
        prob.I_eps_array[7, 5] *= 2.0 ** 40
        prob.I_eps_array[3, 17] *= 2.0 ** 21
    elif kind == "tiny-ieps":
        prob.I_eps_array *= 2.0 ** -110
    else:
        prob.wx_array = np.array([prob.wx_array[0], 1e-7, prob.wx_array[2]])
    if per_band:
        # the same three frequencies stored once per band (stride 3), shifted per band
        wxb = np.repeat(prob.wx_array[None, :], prob.number_bands, 0)
        wxb[:, [0, 2]] += np.linspace(-0.3, 0.3, prob.number_bands)[:, None]
        wxb = np.ascontiguousarray(wxb).reshape(-1)
        o = O.gpp(W.GppProblem(**{**prob.__dict__, "wx_array": wxb}), wx_band_stride=3)
        g = _run_plan(sigma_lib, prob, 0, wx=wxb, wx_stride=3)[0]
    else:
        o = O.gpp(prob)
        g = sigma_lib.gpp_host(prob, 0)
    for x in g:
        assert np.all(np.isfinite(x))
    assert np.any(o[1] != 0)
    _check(g, o, 0)


def test_invalid_indices_are_errors(sigma_lib):
    prob = W.gpp_random(4, 1, 256, 8, 22)
    prob.inv_igp_index = prob.inv_igp_index.copy()
    prob.inv_igp_index[2] = 257  # indigp > ncouls: the reference reads indinv out of bounds
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.gpp_host(prob, 0)
    assert e.value.status == -2
    prob = W.gpp_random(4, 1, 256, 8, 22)
    prob.indinv = prob.indinv.copy()
    prob.indinv[prob.inv_igp_index[1]] = 256  # igp == ncouls: aqsmtemp / vcoul read past the end
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.gpp_host(prob, 1)
    assert e.value.status == -2
    prob = W.gpp_random(4, 5, 256, 8, 22)   # nvband > number_bands
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.gpp_host(prob, 0)
    assert e.value.status == -1


def _to_dev(a):
    a = np.ascontiguousarray(a)
    if np.iscomplexobj(a):
        a = a.view(np.float64)
    return torch.from_numpy(a.copy()).cuda()


def _run_plan(S, prob, prec, wx=None, wx_stride=0, reps=1):
    plan = S.GppPlan(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, prob.inv_igp_index,
                     prob.indinv, precision=prec)
    d = [_to_dev(x) for x in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array,
                              prob.vcoul)]
    dwx = _to_dev(prob.wx_array if wx is None else wx)
    outs = []
    for _ in range(reps):
        ach = torch.zeros(6, dtype=torch.float64, device="cuda")
        asx = torch.zeros_like(ach)
        n1 = torch.zeros(2 * prob.number_bands, dtype=torch.float64, device="cuda")
        plan.execute(dwx, *d, ach, asx, n1, occ=prob.occ, wx_band_stride=wx_stride)
        torch.cuda.synchronize()
        outs.append(tuple(t.cpu().numpy().view(np.complex128) for t in (ach, asx, n1)))
    plan.close()
    return outs


@pytest.mark.parametrize("stress", [False, True], ids=["random", "stress"])
@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_per_band_frequencies(sigma_lib, prec, stress):
    # frequencies that differ per band (ekq(n1) of the Fortran original,
    # gppkernel.deslippe.09.30.2014.f90:238): wx_array[n1][3], stride 3
    prob = W.gpp_random(37, 3, 900, 29, 23, stress=stress)
    rng = np.random.default_rng(0)
    wxb = np.repeat(prob.wx_array[None, :], prob.number_bands, 0) + rng.uniform(-0.7, 0.7, (prob.number_bands, 1))
    wxb = np.ascontiguousarray(wxb)
    o = O.gpp(W.GppProblem(**{**prob.__dict__, "wx_array": wxb.reshape(-1)}), wx_band_stride=3)
    g = _run_plan(sigma_lib, prob, prec, wx=wxb.reshape(-1), wx_stride=3)[0]
    _check(g, o, prec)


def test_per_band_frequencies_long_g_sums(sigma_lib):
    """Per-band frequencies with 16384 g-vectors per column (items summing
    thousands of float-float terms), FP64 at the 1e-12 bar."""
    prob = W.gpp_random(64, 2, 16384, 160, 29)
    rng = np.random.default_rng(2)
    wxb = np.repeat(prob.wx_array[None, :], prob.number_bands, 0) + rng.uniform(-0.6, 0.6, (prob.number_bands, 1))
    wxb = np.ascontiguousarray(wxb).reshape(-1)
    o = O.gpp(W.GppProblem(**{**prob.__dict__, "wx_array": wxb}), wx_band_stride=3)
    g = _run_plan(sigma_lib, prob, 0, wx=wxb, wx_stride=3)[0]
    _check(g, o, 0)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_per_band_exact_poles_and_guard_edges(sigma_lib, prec):
    """Per-band frequencies with an exact pole of one band's frequency, a
    term exactly on the |wdiff|^2 = 0.25 boundary, a zero wtilde and
    |wtilde|^2 >= 62000 (the guard's second condition binding): the
    per-band pass takes these decisions with the FP64 expressions."""
    prob = W.gpp_random(21, 3, 700, 26, 27)
    rng = np.random.default_rng(1)
    wxb = np.repeat(prob.wx_array[None, :], prob.number_bands, 0) + rng.uniform(-0.5, 0.5, (prob.number_bands, 1))
    prob.wtilde_array = prob.wtilde_array.copy()
    prob.wtilde_array[2, 10] = complex(wxb[4, 0], 0.0)        # exact pole of band 4
    prob.wtilde_array[5, 11] = complex(wxb[17, 2], 0.0)       # exact pole of band 17
    prob.wtilde_array[7, 12] = complex(wxb[9, 1] + 0.5, 0.0)  # |wdiff|^2 = 0.25 for band 9
    prob.wtilde_array[8, 13] = 0.0
    prob.wtilde_array[9, 14] = complex(300.0, 0.5)
    wxb = np.ascontiguousarray(wxb).reshape(-1)
    o = O.gpp(W.GppProblem(**{**prob.__dict__, "wx_array": wxb}), wx_band_stride=3)
    g = _run_plan(sigma_lib, prob, prec, wx=wxb, wx_stride=3)[0]
    for x in g:
        assert np.all(np.isfinite(x))
    _check(g, o, prec)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_frequencies_not_exact_in_fp32(sigma_lib, prec):
    # shared frequencies with a low part below FP32 precision (the mixed path
    # then carries wx as an FP32 hi/lo pair)
    prob = W.gpp_random(30, 2, 1500, 40, 25)
    prob.wx_array = np.array([3.1, 4.2 + 1e-9, 5.3])
    o = O.gpp(prob)
    g = _run_plan(sigma_lib, prob, prec)[0]
    _check(g, o, prec)


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_bitwise_repeatable(sigma_lib, prec):
    prob = W.gpp_random(50, 2, 3000, 75, 24, stress=True)
    outs = _run_plan(sigma_lib, prob, prec, reps=3)
    for r in outs[1:]:
        for x, y in zip(outs[0], r):
            assert np.array_equal(x, y)


def test_device_fill_matches_host_generator(sigma_lib):
    n = 100_003
    t = torch.empty(2 * n, dtype=torch.float64, device="cuda")
    sigma_lib.fill_complex_device(t.data_ptr(), n, 9, W.AID_WTILDE, (0.5, 5.0), (-0.1, 0.1))
    h = W.fill_complex(9, W.AID_WTILDE, n, (0.5, 5.0), (-0.1, 0.1))
    assert np.array_equal(t.cpu().numpy(), h.view(np.float64))
    r = torch.empty(n, dtype=torch.float64, device="cuda")
    sigma_lib.fill_real_device(r.data_ptr(), n, 9, W.AID_VCOUL, 0.1, 10.0)
    assert np.array_equal(r.cpu().numpy(), W.fill_real(9, W.AID_VCOUL, n, 0.1, 10.0))
    sigma_lib.fill_stress_device(t.data_ptr(), n, 9, W.AID_STRESS, W.wx_frequencies())
    W.stress_wtilde(h, W.wx_frequencies(), 9)
    assert np.array_equal(t.cpu().numpy(), h.view(np.float64))


# ------------------------------------------------------------ production shape
class Production:
    """512 bands, nvband 2, ncouls 32768, ngpown 1638 (512 2 32768 20), seeded
    fill generated on the device; host copies made on demand."""

    def __init__(self, S, seed, stress=False):
        nb, nc = 512, 32768
        ng = nc // 20
        self.nb, self.nvb, self.nc, self.ng = nb, 2, nc, ng
        self.aqsm = torch.empty(2 * nb * nc, dtype=torch.float64, device="cuda")
        self.aqsn = torch.empty_like(self.aqsm)
        self.ieps = torch.empty(2 * ng * nc, dtype=torch.float64, device="cuda")
        self.wt = torch.empty_like(self.ieps)
        self.vcoul = torch.empty(nc, dtype=torch.float64, device="cuda")
        S.fill_complex_device(self.aqsm.data_ptr(), nb * nc, seed, W.AID_AQSM, (-1, 1), (-1, 1))
        S.fill_complex_device(self.aqsn.data_ptr(), nb * nc, seed, W.AID_AQSN, (-1, 1), (-1, 1))
        S.fill_complex_device(self.ieps.data_ptr(), ng * nc, seed, W.AID_IEPS, (-1, 1), (-1, 1))
        S.fill_complex_device(self.wt.data_ptr(), ng * nc, seed, W.AID_WTILDE, (0.5, 5.0), (-0.1, 0.1))
        if stress:
            S.fill_stress_device(self.wt.data_ptr(), ng * nc, seed, W.AID_STRESS, W.wx_frequencies())
        S.fill_real_device(self.vcoul.data_ptr(), nc, seed, W.AID_VCOUL, 0.1, 10.0)
        self.inv, self.indinv = W.gpp_index_maps(nc, ng)
        self.wx = torch.tensor(W.wx_frequencies(), dtype=torch.float64, device="cuda")
        self.S = S

    def run(self, prec, aqsn=None):
        plan = self.S.GppPlan(self.nb, self.nvb, self.nc, self.ng, self.inv, self.indinv, precision=prec)
        ach = torch.zeros(6, dtype=torch.float64, device="cuda")
        asx = torch.zeros_like(ach)
        n1 = torch.zeros(2 * self.nb, dtype=torch.float64, device="cuda")
        plan.execute(self.wx, self.aqsm, self.aqsn if aqsn is None else aqsn, self.ieps, self.wt,
                     self.vcoul, ach, asx, n1)
        torch.cuda.synchronize()
        plan.close()
        return tuple(t.cpu().numpy().view(np.complex128) for t in (ach, asx, n1))

    def host_problem(self):
        c = lambda t, r: t.cpu().numpy().view(np.complex128).reshape(r, self.nc)
        return W.GppProblem(self.nb, self.nvb, self.nc, self.ng, self.inv, self.indinv,
                            W.wx_frequencies(), c(self.aqsm, self.nb), c(self.aqsn, self.nb),
                            c(self.ieps, self.ng), c(self.wt, self.ng), self.vcoul.cpu().numpy())


@pytest.fixture(scope="module")
def production(sigma_lib):
    p = Production(sigma_lib, W.GPP_PRODUCTION_SEED)
    yield p
    del p
    torch.cuda.empty_cache()


def test_production_sampled_bands_match_oracle(production):
    g = production.run(0)
    prob = production.host_problem()
    for band in (0, 1, 300, 511):  # two occupied, two not
        _, _, on1 = O.gpp(prob, band, band + 1)
        assert rel_err(g[2][band], on1[band]) <= FP64_TOL
    # acht_n1_loc sums to achtemp[2]
    assert abs(g[2].sum() - g[0][2]) / abs(g[0][2]) <= 1e-13


def test_production_mixed_within_bar_of_fp64(production):
    g64 = production.run(0)
    gmx = production.run(1)
    assert rel_err(gmx[0], g64[0]).max() <= MIXED_TOL
    assert rel_err(gmx[1], g64[1]).max() <= MIXED_TOL
    assert normwise_err(gmx[2], g64[2]) <= MIXED_TOL


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_production_linearity_in_aqsn(production, prec):
    # every output is linear in aqsn; scaling by 2 is exact in both precisions
    base = production.run(prec)
    doubled = production.run(prec, aqsn=production.aqsn * 2.0)
    for x, y in zip(base, doubled):
        assert np.array_equal(2.0 * x, y)


def test_production_stress_mixed_within_bar(sigma_lib):
    p = Production(sigma_lib, W.GPP_STRESS_SEED, stress=True)
    g64 = p.run(0)
    gmx = p.run(1)
    del p
    torch.cuda.empty_cache()
    assert rel_err(gmx[0], g64[0]).max() <= MIXED_TOL
    assert rel_err(gmx[1], g64[1]).max() <= MIXED_TOL


# ------------------------------------------------------------ tensor-core form
TENSOR_CASES = [c for c in RANDOM_CASES if c[3] >= 20] + [
    (50, 2, 2080, 128, 31, False),      # 3 x 128 contraction rows: no padding rows to zero
    (24, 0, 1000, 128, 32, True),       # the same with a ragged last K tile and no occupied band
    # more columns and g-vectors: several factor items per column block and
    # several contraction K splits
    (40, 3, 8192, 300, 33, False),
    (37, 2, 8000, 300, 34, True),       # ragged last K tile, stress fill
]


@pytest.mark.parametrize("case", TENSOR_CASES, ids=lambda c: f"nb{c[0]}-nv{c[1]}-nc{c[2]}-ng{c[3]}{'-stress' if c[5] else ''}")
def test_tensor_random_matches_oracle(sigma_lib, case):
    """Split-BF16 tensor-core band sum: the same error model as the FP32
    path (terms carry FP32-level relative errors)."""
    nb, nvb, nc, ng, seed, stress = case
    prob = W.gpp_random(nb, nvb, nc, ng, seed, stress=stress)
    o = O.gpp(prob)
    g = sigma_lib.gpp_host(prob, sigma_lib.PREC_TENSOR)
    _check(g, o, 1, abs2=O.gpp_abs2(prob))


def test_tensor_constant_fill_and_limits(sigma_lib):
    prob = W.gpp_constant(128, 2, 8192, 20)
    o = O.gpp(prob)
    g = sigma_lib.gpp_host(prob, sigma_lib.PREC_TENSOR)
    _check(g, o, 1)
    # per-band frequencies have no shared factor: the tensor form refuses them
    prob = W.gpp_random(37, 3, 900, 29, 23)
    wxb = np.ascontiguousarray(np.repeat(prob.wx_array[None, :], prob.number_bands, 0)).reshape(-1)
    with pytest.raises(sigma_lib.SigmaError) as e:
        _run_plan(sigma_lib, prob, sigma_lib.PREC_TENSOR, wx=wxb, wx_stride=3)
    assert e.value.status == -8
    # fewer than ~18 columns: more frequency segments per tile than the kernel holds
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.gpp_host(W.gpp_random(7, 1, 333, 5, 14), sigma_lib.PREC_TENSOR)
    assert e.value.status == -8


def test_production_tensor_within_bar_of_fp64(production):
    g64 = production.run(0)
    gtc = production.run(2)
    assert rel_err(gtc[0], g64[0]).max() <= MIXED_TOL
    assert rel_err(gtc[1], g64[1]).max() <= MIXED_TOL
    assert normwise_err(gtc[2], g64[2]) <= MIXED_TOL


def test_mixed_checked_reports_its_error(sigma_lib):
    """sigma_gpp_mixed_checked: the mixed outputs plus rel_err_out[6], the
    relative error of each achtemp / asxtemp against the FP64 form."""
    prob = W.gpp_random(40, 3, 2048, 100, 44, stress=True)
    lib = sigma_lib.load()
    inv = np.ascontiguousarray(prob.inv_igp_index, np.int32)
    indinv = np.ascontiguousarray(prob.indinv, np.int32)
    c = lambda a: np.ascontiguousarray(a, np.complex128)
    ins = [c(prob.aqsmtemp), c(prob.aqsntemp), c(prob.I_eps_array), c(prob.wtilde_array)]
    vc = np.ascontiguousarray(prob.vcoul, np.float64)
    wx = np.ascontiguousarray(prob.wx_array, np.float64)
    ach, asx = np.zeros(3, np.complex128), np.zeros(3, np.complex128)
    err = np.full(6, -1.0)
    st = lib.sigma_gpp_mixed_checked(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, 0, 3,
                                     inv.ctypes.data, indinv.ctypes.data, wx.ctypes.data, 1.0,
                                     *[a.ctypes.data for a in ins], vc.ctypes.data, ach.ctypes.data,
                                     asx.ctypes.data, None, None, err.ctypes.data)
    assert st == 0
    g64 = sigma_lib.gpp_host(prob, sigma_lib.PREC_FP64)
    gmx = sigma_lib.gpp_host(prob, sigma_lib.PREC_MIXED)
    assert np.array_equal(ach, gmx[0]) and np.array_equal(asx, gmx[1])
    expect = np.concatenate([rel_err(gmx[0], g64[0]), rel_err(gmx[1], g64[1])])
    assert np.allclose(err, expect, rtol=1e-12, atol=0)
    assert err.max() <= MIXED_TOL
