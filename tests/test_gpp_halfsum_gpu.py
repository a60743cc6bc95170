"""gppsum = 1 ("half sum") GPP (sigma_gpp_halfsum_*) on the GPU against the
oracle's restatement of gppKerSeq.cpp (pinned to that driver's printed
achtemp and to its own solvers in tests/test_oracle.py).

Bar: FP64, every achtemp / asxtemp / achstemp output within 1e-12 relative of
the oracle; acht_n1_loc within 1e-12 of its largest entry.  The host entry
takes gppKerSeq.cpp's g-vector-major layout; the device plan is tested in
both layouts.
"""
import json
import pathlib

import numpy as np
import pytest
import torch

import workload as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-12

CASES = [
    # number_bands, nvband, ncouls, ngpown, seed, stress
    (40, 3, 2048, 100, 71, False),
    (37, 2, 1536, 33, 72, False),     # igp on 512 and 1024: the unpaired igp term
    (33, 1, 1100, 37, 73, True),      # ragged, near-pole wtilde
    (7, 0, 333, 5, 74, False),        # no occupied band
    (9, 9, 777, 21, 75, False),       # every band occupied
    (70, 5, 4096, 130, 76, True),     # several band and column blocks, occupied group of 5
]


def _rel_ok(g, o, tol=TOL):
    return np.all(np.abs(g - o) <= tol * np.maximum(np.abs(o), 1e-300))


def _check(g, o, nvb):
    ach, asx, n1, stat = g
    assert _rel_ok(ach, o[0]), (ach, o[0])
    if nvb:
        assert _rel_ok(asx, o[1]), (asx, o[1])
    else:
        assert np.all(asx == 0)
    assert np.abs(n1 - o[2]).max() <= TOL * np.abs(o[2]).max()
    if stat is not None:
        assert abs(stat - o[3]) <= TOL * abs(o[3])


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:4])) + ("s" if c[5] else ""))
def test_halfsum_host_matches_oracle(sigma_lib, case):
    nb, nvb, nc, ng, seed, stress = case
    p = W.gpp_random(nb, nvb, nc, ng, seed, stress=stress)
    o = O.gpp_halfsum(p)
    _check(sigma_lib.gpp_halfsum_host(p), o, nvb)


def test_halfsum_constant_fill_matches_reference_driver(sigma_lib):
    ref = json.loads((pathlib.Path(__file__).parent / "golden" / "gpp_halfsum_reference.json").read_text())
    for run in ref["runs"]:
        g = sigma_lib.gpp_halfsum_host(W.gpp_constant(*run["shape"]))
        r = np.array([complex(*z) for z in run["achtemp"]])
        if np.all(r == 0):
            assert np.all(g[0] == 0)
        else:
            assert np.all(np.abs(g[0] - r) <= 1e-12 * np.abs(r))


def _device(p, gvec_major):
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a.T if gvec_major else a)).view(torch.float64).cuda()
    return dict(aqsm=t(p.aqsmtemp), aqsn=t(p.aqsntemp), ieps=t(p.I_eps_array), wt=t(p.wtilde_array),
                vcoul=torch.from_numpy(p.vcoul.copy()).cuda(),
                wx=torch.from_numpy(p.wx_array[:3].copy()).cuda())


@pytest.mark.parametrize("gvec_major", [False, True], ids=["band_major", "gvec_major"])
def test_halfsum_plan_layouts_and_repeatability(sigma_lib, gvec_major):
    nb, nvb, nc, ng = 45, 3, 2560, 96
    p = W.gpp_random(nb, nvb, nc, ng, 77)
    o = O.gpp_halfsum(p)
    flags = sigma_lib.HALFSUM_STATIC | (sigma_lib.HALFSUM_GVEC_MAJOR if gvec_major else 0)
    plan = sigma_lib.GppHalfSumPlan(nb, nvb, nc, ng, p.inv_igp_index, p.indinv, flags=flags)
    d = _device(p, gvec_major)
    outs = []
    for _ in range(2):
        ach, asx = torch.zeros(6, dtype=torch.float64, device="cuda"), torch.zeros(6, dtype=torch.float64,
                                                                                    device="cuda")
        n1 = torch.zeros(2 * nb, dtype=torch.float64, device="cuda")
        st = torch.zeros(2, dtype=torch.float64, device="cuda")
        plan.execute(d["wx"], d["aqsm"], d["aqsn"], d["ieps"], d["wt"], d["vcoul"], ach, asx, n1, st)
        torch.cuda.synchronize()
        outs.append(torch.cat([ach, asx, n1, st]).cpu().numpy())
    plan.close()
    assert np.array_equal(outs[0], outs[1])          # fixed-order sums: bit-identical
    v = outs[0].view(np.complex128)
    _check((v[0:3], v[3:6], v[6:6 + nb], v[6 + nb]), o, nvb)


def test_halfsum_without_static(sigma_lib):
    p = W.gpp_random(12, 2, 700, 30, 78)
    o = O.gpp_halfsum(p)
    g = sigma_lib.gpp_halfsum_host(p, want_static=False, want_n1=False)
    assert _rel_ok(g[0], o[0]) and _rel_ok(g[1], o[1])
    # achstemp asked of a plan made without the static flag
    plan = sigma_lib.GppHalfSumPlan(12, 2, 700, 30, p.inv_igp_index, p.indinv, flags=0)
    d = _device(p, False)
    z = lambda n: torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(sigma_lib.SigmaError) as e:
        plan.execute(d["wx"], d["aqsm"], d["aqsn"], d["ieps"], d["wt"], d["vcoul"], z(6), z(6), None, z(2))
    assert e.value.status == -8
    plan.close()


def test_halfsum_skipped_column_and_omega_cut(sigma_lib):
    """A column the reference skips (igp < 0) and an occupied-band column whose
    loop stops early at a small Omega2 (gppKerSeq.cpp:96)."""
    p = W.gpp_random(10, 3, 900, 30, 79)
    p.indinv = p.indinv.copy()
    p.indinv[p.inv_igp_index[4]] = -1
    p.I_eps_array = p.I_eps_array.copy()
    p.I_eps_array[7, 100] = 1e-9          # |Omega2| < to1 at ig = 100 of column 7
    o = O.gpp_halfsum(p)
    _check(sigma_lib.gpp_halfsum_host(p), o, 3)


def test_halfsum_config0_shape_random(sigma_lib):
    """The mini-app's small shape (128 x 8192 x 409) with seeded random inputs."""
    p = W.gpp_random(128, 2, 8192, 409, 80)
    o = O.gpp_halfsum(p)
    _check(sigma_lib.gpp_halfsum_host(p), o, 2)


# ---- tensor-core form (SIGMA_HALFSUM_TENSOR): band sums as split-BF16
# contractions, FP32-class error; against the FP64 form (itself pinned above)
TENSOR_CASES = [
    (40, 3, 2048, 100, 81, False),
    (37, 2, 1536, 33, 82, True),      # unpaired igp terms, near-pole wtilde
    (70, 0, 4096, 130, 83, False),    # no occupied band
    (30, 2, 1000, 128, 84, False),    # contraction rows a multiple of 128 (no padding), ragged K
    (45, 5, 2048, 64, 85, True),      # three occupied-band groups, 192 slab rows
]


@pytest.mark.parametrize("case", TENSOR_CASES, ids=lambda c: "x".join(map(str, c[:4])) + ("s" if c[5] else ""))
def test_halfsum_tensor_matches_fp64(sigma_lib, case):
    nb, nvb, nc, ng, seed, stress = case
    p = W.gpp_random(nb, nvb, nc, ng, seed, stress=stress)
    f = sigma_lib.gpp_halfsum_host(p)
    t = sigma_lib.gpp_halfsum_host(p, tensor=True)
    rel = lambda a, b: np.abs(a - b) / np.abs(b)
    assert np.all(rel(t[0], f[0]) <= 2e-6), rel(t[0], f[0])
    if nvb:
        # occupied bands: float-float factors, FP32 products, float-float sums
        assert np.all(rel(t[1], f[1]) <= 1e-6), rel(t[1], f[1])
        assert np.all(rel(t[2][:nvb], f[2][:nvb]) <= 1e-6), rel(t[2][:nvb], f[2][:nvb])
    assert rel(t[3], f[3]) <= 2e-6
    assert np.linalg.norm(t[2] - f[2]) <= 1e-6 * np.linalg.norm(f[2])


# ---- production shape: 512 bands, nvband 2, ncouls 32768, ngpown 1638
@pytest.fixture(scope="module")
def production_half(sigma_lib):
    nb, nvb, nc = 512, 2, 32768
    ng = nc // 20
    seed = W.GPP_PRODUCTION_SEED
    f64 = dict(dtype=torch.float64, device="cuda")
    d = dict(aqsm=torch.empty(2 * nb * nc, **f64), aqsn=torch.empty(2 * nb * nc, **f64),
             ieps=torch.empty(2 * ng * nc, **f64), wt=torch.empty(2 * ng * nc, **f64),
             vcoul=torch.empty(nc, **f64), wx=torch.tensor(W.wx_frequencies(), **f64))
    sigma_lib.fill_complex_device(d["aqsm"].data_ptr(), nb * nc, seed, W.AID_AQSM, (-1, 1), (-1, 1))
    sigma_lib.fill_complex_device(d["aqsn"].data_ptr(), nb * nc, seed, W.AID_AQSN, (-1, 1), (-1, 1))
    sigma_lib.fill_complex_device(d["ieps"].data_ptr(), ng * nc, seed, W.AID_IEPS, (-1, 1), (-1, 1))
    sigma_lib.fill_complex_device(d["wt"].data_ptr(), ng * nc, seed, W.AID_WTILDE, (0.5, 5.0), (-0.1, 0.1))
    sigma_lib.fill_real_device(d["vcoul"].data_ptr(), nc, seed, W.AID_VCOUL, 0.1, 10.0)
    inv, indinv = W.gpp_index_maps(nc, ng)
    outs = {}
    for name, flags in (("fp64", sigma_lib.HALFSUM_STATIC),
                        ("tensor", sigma_lib.HALFSUM_STATIC | sigma_lib.HALFSUM_TENSOR)):
        plan = sigma_lib.GppHalfSumPlan(nb, nvb, nc, ng, inv, indinv, flags=flags)
        z = lambda n: torch.zeros(n, **f64)
        ach, asx, n1, st = z(6), z(6), z(2 * nb), z(2)
        plan.execute(d["wx"], d["aqsm"], d["aqsn"], d["ieps"], d["wt"], d["vcoul"], ach, asx, n1, st)
        torch.cuda.synchronize()
        plan.close()
        outs[name] = [t.cpu().numpy().view(np.complex128).copy() for t in (ach, asx, n1, st)]
    c = lambda t, r: t.cpu().numpy().view(np.complex128).reshape(r, nc)
    prob = W.GppProblem(nb, nvb, nc, ng, inv, indinv, W.wx_frequencies(), c(d["aqsm"], nb), c(d["aqsn"], nb),
                        c(d["ieps"], ng), c(d["wt"], ng), d["vcoul"].cpu().numpy())
    del d
    torch.cuda.empty_cache()
    return outs, prob


def test_halfsum_production_sampled_bands_match_oracle(production_half):
    outs, prob = production_half
    g = outs["fp64"]
    for band in (0, 1, 300, 511):  # two occupied, two not
        _, _, on1, _ = O.gpp_halfsum(prob, band_begin=band, band_end=band + 1)
        assert abs(g[2][band] - on1[band]) <= TOL * abs(on1[band])
    assert abs(g[2].sum() - g[0][2]) <= 1e-13 * np.abs(g[2]).sum()   # acht_n1_loc sums to achtemp[2]


def test_halfsum_production_tensor_within_bar_of_fp64(production_half):
    outs, _ = production_half
    f, t = outs["fp64"], outs["tensor"]
    rel = lambda a, b: np.abs(a - b) / np.abs(b)
    assert np.all(rel(t[0], f[0]) <= 2e-6)
    assert np.all(rel(t[1], f[1]) <= 1e-6)        # occupied bands: float-float factors, FP32 products
    assert np.all(rel(t[2][:2], f[2][:2]) <= 1e-6)
    assert rel(t[3], f[3]) <= 2e-6
    assert np.linalg.norm(t[2] - f[2]) <= 1e-6 * np.linalg.norm(f[2])
