"""The CPU oracle pinned against the reference's own outputs and closed forms.

Fixtures in tests/golden/ come from the reference itself
(tests/golden/make_golden.py): the unmodified BGW-Kernels/gppKer.cpp driver's
printed achtemp on the constant fill, and its flagOCC_solver's per-column
sums on seeded inputs.
"""
import json
import pathlib

import numpy as np
import pytest

import workload as W
from conftest import rel_err
from oracle import oracle as O

GOLD = pathlib.Path(__file__).resolve().parent / "golden"


def _igp_map(prob):
    return np.array([prob.ncouls - 1 if i == prob.ncouls else int(prob.indinv[i])
                     for i in prob.inv_igp_index], dtype=np.int32)


@pytest.mark.parametrize("run", json.loads((GOLD / "gpp_reference_constfill.json").read_text())["runs"],
                         ids=lambda r: f"{'x'.join(map(str, r['shape']))}-t{r['omp_threads']}")
def test_oracle_matches_reference_driver_constant_fill(run):
    nb, nvb, nc, npg = run["shape"]
    if nb * nc * (nc // npg) > 2e8:
        pytest.skip("large constant-fill shape checked in the slow tier")
    prob = W.gpp_constant(nb, nvb, nc, npg)
    ach, asx, n1 = O.gpp(prob)
    ref = np.array([complex(*z) for z in run["achtemp"]])
    exact = np.array([complex(*z) for z in run["closed_form_achtemp"]])
    exact_asx = np.array([complex(*z) for z in run["closed_form_asxtemp"]])
    # the oracle's compensated sums sit on the closed form ...
    assert rel_err(ach, exact).max() < 1e-15
    assert rel_err(asx, exact_asx).max() < 1e-15
    # ... and the reference's printed values within its own rounding (15 digits,
    # plain OpenMP sums: up to ~1e-12 relative at these shapes)
    assert rel_err(ref, ach).max() < 2e-12
    # acht_n1_loc sums to achtemp[2]
    assert abs(n1.sum() - ach[2]) / abs(ach[2]) < 1e-14


def test_oracle_production_constant_fill_closed_form():
    # the largest golden shape (config 128 2 8192 20), compensated oracle vs exact
    runs = json.loads((GOLD / "gpp_reference_constfill.json").read_text())["runs"]
    run = [r for r in runs if r["shape"] == [128, 2, 8192, 20]][0]
    prob = W.gpp_constant(128, 2, 8192, 20)
    ach, asx, _ = O.gpp(prob)
    exact = np.array([complex(*z) for z in run["closed_form_achtemp"]])
    ref = np.array([complex(*z) for z in run["achtemp"]])
    assert rel_err(ach, exact).max() < 1e-15
    assert rel_err(ref, exact).max() < 2e-12


@pytest.mark.parametrize("name", ["random_a", "random_b", "stress_a"])
def test_oracle_terms_match_reference_flagocc(name):
    g = np.load(GOLD / f"gpp_flagocc_{name}.npz")
    nb, nc, ng, seed, stress = (int(x) for x in g["meta"])
    prob = W.gpp_random(nb, nb, nc, ng, seed, stress=bool(stress))
    sch, ssx = O.gpp_columns(prob)
    scale_sch = np.abs(g["sch"]).max()
    scale_ssx = np.abs(g["ssx"]).max()
    assert np.abs(sch - g["sch"]).max() / scale_sch < 1e-13
    assert np.abs(ssx - g["ssx"]).max() / scale_ssx < 1e-13


def test_oracle_unoccupied_term_equals_occupied_sch():
    # achtemp semantics are uniform over bands: the hot-loop term
    # (gppKer.cpp:396-407) and flagOCC's sch (:38-40, :64) agree
    prob = W.gpp_random(4, 0, 300, 11, 5)
    sch_unocc, _ = O.gpp_columns(prob)
    prob.nvband = 4
    sch_occ, _ = O.gpp_columns(prob)
    assert np.abs(sch_unocc - sch_occ).max() / np.abs(sch_occ).max() < 1e-14


def test_port_agrees_with_compensated_oracle():
    prob = W.gpp_random(12, 2, 1536, 60, 3)
    a1, s1, n1 = O.gpp(prob)
    a2, s2, n2 = O.gpp(prob, port=True)
    assert rel_err(a2, a1).max() < 1e-12
    assert rel_err(s2, s1).max() < 1e-12
    assert np.abs(n2 - n1).max() / np.abs(n1).max() < 1e-12


def test_oracle_thread_count_independent():
    prob = W.gpp_random(6, 2, 777, 19, 4, stress=True)
    r1 = O.gpp(prob, nthreads=1)
    r4 = O.gpp(prob, nthreads=4)
    for x, y in zip(r1, r4):
        assert np.array_equal(x, y)


def test_oracle_band_ranges_sum():
    prob = W.gpp_random(10, 3, 512, 16, 9)
    full = O.gpp(prob)
    a = O.gpp(prob, 0, 4)
    b = O.gpp(prob, 4, 10)
    assert rel_err(a[0] + b[0], full[0]).max() < 1e-14
    assert rel_err(a[1] + b[1], full[1]).max() < 1e-14
    assert np.array_equal(full[2][:4], a[2][:4]) and np.array_equal(full[2][4:], b[2][4:])


def test_oracle_rejects_reference_out_of_bounds_indices():
    prob = W.gpp_random(2, 1, 64, 4, 1)
    prob.inv_igp_index = np.array([0, 1, 65, 3], np.int32)  # indigp > ncouls
    with pytest.raises(O.OracleError):
        O.gpp(prob)
    prob.inv_igp_index = np.array([0, 1, 2, 3], np.int32)
    prob.indinv = np.arange(64, dtype=np.int32)
    prob.indinv[2] = 64  # igp == ncouls: the reference reads past the row
    with pytest.raises(O.OracleError):
        O.gpp(prob)


def test_oracle_skips_columns_like_reference():
    # igp < 0 or igp > ncouls: the column is skipped (gppKer.cpp:328)
    prob = W.gpp_random(3, 1, 64, 4, 2)
    prob.indinv = prob.indinv.copy()
    target = prob.inv_igp_index[1]
    prob.indinv[target] = -5
    sch, _ = O.gpp_columns(prob)
    assert np.all(sch[:, 1, :] == 0)
    ach, _, _ = O.gpp(prob)
    ach_ref = np.zeros(3, complex)
    for my_igp in (0, 2, 3):
        igp = prob.ncouls - 1 if prob.inv_igp_index[my_igp] == prob.ncouls else prob.indinv[prob.inv_igp_index[my_igp]]
        ach_ref += (sch[:, my_igp, :] * prob.vcoul[igp]).sum(axis=0)
    assert rel_err(ach, ach_ref).max() < 1e-13


def test_oracle_exact_pole_is_dropped():
    # wtilde == wx exactly: |wdiff|^2 = 0, the reference's delw is NaN and the
    # guard drops the term; ssx is 0 (its delwr > to1 test is false for NaN)
    prob = W.gpp_random(2, 2, 128, 8, 6)
    prob.wtilde_array = prob.wtilde_array.copy()
    prob.wtilde_array[3, 5] = complex(prob.wx_array[1], 0.0)
    ach, asx, n1 = O.gpp(prob)
    assert np.all(np.isfinite(ach)) and np.all(np.isfinite(asx)) and np.all(np.isfinite(n1))


def test_ff_oracle_matches_matmul_and_closed_form():
    p = W.ff_random(5, 257, 7, 3, 4)
    out = O.ff_schdt(p)
    igp = p.indinv[p.inv_igp_index]
    tempz = np.einsum("fgi,ni->fgn", p.I_epsR, p.aqsntemp)
    ref = np.einsum("fgn,ng->nf", tempz, np.conj(p.aqsmtemp[:, igp]))
    assert np.abs(out.reshape(5, 3) - ref).max() / np.abs(ref).max() < 1e-13
    c = W.ff_constant(4, 100, 6, 2)
    outc = O.ff_schdt(c).reshape(4, 2)
    exact = 6 * 100 * 0.5 * (0.5 + 0.5j)
    assert np.abs(outc - exact).max() / abs(exact) < 1e-15


def _achstemp_numpy(p):
    igp = _igp_map(p)
    ok = (igp >= 0) & (igp <= p.ncouls)
    M = p.aqsntemp @ p.I_eps_array.T                       # sum_ig aqsn[n1][ig] I_eps[my_igp][ig]
    w = np.where(ok, -0.5 * p.vcoul[np.clip(igp, 0, p.ncouls - 1)], 0.0)
    am = np.conj(p.aqsmtemp[:, np.clip(igp, 0, p.ncouls - 1)])
    return (w[None, :] * am * M).sum(axis=1)


def test_static_remainder_oracle_closed_form_and_matmul():
    # gppkernel.deslippe.09.30.2014.f90:195-228 on the constant fill: every
    # term is -0.5 * |0.5+0.5i|^2 * (0.5+0.5i) = -0.125-0.125i
    c = W.gpp_constant(16, 2, 1024, 8)
    tot, n1 = O.gpp_achstemp(c)
    exact = c.number_bands * c.ngpown * c.ncouls * (-0.125 - 0.125j)
    assert tot == exact
    assert np.all(n1 == exact / c.number_bands)
    p = W.gpp_random(9, 1, 700, 31, 12)
    p.indinv = p.indinv.copy()
    p.indinv[p.inv_igp_index[4]] = -3                     # a skipped column
    tot, n1 = O.gpp_achstemp(p)
    ref = _achstemp_numpy(p)
    assert np.abs(n1 - ref).max() / np.abs(ref).max() < 1e-13
    assert abs(tot - ref.sum()) / abs(tot) < 1e-13


FF_REF = json.loads((GOLD / "ff_sigma_reference.json").read_text())


@pytest.mark.parametrize("run", FF_REF["constant_fill"], ids=lambda r: "x".join(map(str, r["shape"])))
def test_ff_sigma_oracle_matches_reference_driver_constant_fill(run):
    """The unmodified FFKer_cori/ffKernel.cpp driver's printed results on its
    constant fill (its schDt_matrix stays zero, as in the Fortran)."""
    p = W.ff_sigma_constant(*run["shape"])
    o = O.ff_sigma(p)
    for key, ours in (("achsDtemp", o["achsDtemp"]), ("asxDtemp", o["asxDtemp"][0]),
                      ("achDtemp_cor", o["achDtemp_cor"][0])):
        ref = complex(*run[key])
        assert abs(ours - ref) <= 1e-6 + 1e-12 * abs(ref)   # the driver prints 6 decimals


@pytest.mark.parametrize("case", FF_REF["random"], ids=lambda c: c["name"])
def test_ff_sigma_oracle_matches_reference_kernels(case):
    """The reference's own achsDtemp / asxDtemp / achDtemp_cor kernels on
    seeded inputs (see tests/golden/make_golden.py for the C++ deviations the
    case avoids)."""
    p = W.ff_sigma_random(*case["args"])
    p.freqevalmin = case["freqevalmin"]
    o = O.ff_sigma(p)
    ach = complex(*case["achsDtemp"])
    assert abs(o["achsDtemp"] - ach) <= 1e-13 * abs(ach)
    for z in case["asxDtemp_iw0"]:
        assert abs(o["asxDtemp"][0] - complex(*z)) <= 1e-13 * abs(complex(*z))
    for z in case["achDtemp_cor_iw0"]:
        assert abs(o["achDtemp_cor"][0] - complex(*z)) <= 1e-13 * abs(complex(*z))


def test_ff_sigma_oracle_schdt_epilogue_is_linear():
    # the CH terms from schDt_matrix are linear in it; doubling it doubles
    # achDtemp and achDtemp_corb and the schDt parts of the other two
    p = W.ff_sigma_random(6, 2, 64, 8, 7, 4, 3)
    rng = np.random.default_rng(5)
    sd = rng.standard_normal((6, 7)) + 1j * rng.standard_normal((6, 7))
    z = O.ff_sigma(p)
    a = O.ff_sigma(p, sd)
    b = O.ff_sigma(p, 2 * sd)
    for k in ("achDtemp", "achDtemp_corb"):
        assert np.all(z[k] == 0)
        assert np.abs(b[k] - 2 * a[k]).max() <= 1e-13 * np.abs(a[k]).max()
    for k in ("achDtemp_cor", "ach2Dtemp"):
        assert np.abs((b[k] - z[k]) - 2 * (a[k] - z[k])).max() <= 1e-12 * np.abs(a[k] - z[k]).max()
    assert a["achsDtemp"] == z["achsDtemp"] and np.array_equal(a["asxDtemp"], z["asxDtemp"])


REAL_REF = json.loads((GOLD / "gpp_real_reference.json").read_text())


@pytest.mark.parametrize("run", REAL_REF["runs"], ids=lambda r: "x".join(map(str, r["shape"])))
def test_real_oracle_matches_reference_driver_constant_fill(run):
    """The unmodified gppKer_real.cpp driver's printed achtemp (15 digits)."""
    ach, _, _ = O.gpp_real(W.gpp_real_constant(*run["shape"]))
    ref = np.array(run["achtemp"])
    assert np.abs(ach - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["real_a", "real_b"])
def test_real_oracle_terms_match_reference_flagocc(name):
    """Per-column sums of the real mini-app's own occupied-band solver; the
    oracle's band totals must equal their vcoul-weighted sum."""
    f = np.load(GOLD / f"gpp_real_flagocc_{name}.npz")
    nb, nc, ng, seed = (int(x) for x in f["meta"])
    p = W.gpp_real_random(nb, nb, nc, ng, seed)
    igp = _igp_map(p)
    ach_ref = (f["sch"] * p.vcoul[igp][None, :, None]).sum(axis=(0, 1))
    asx_ref = (f["ssx"] * p.vcoul[igp][None, :, None]).sum(axis=(0, 1))
    ach, asx, _ = O.gpp_real(p)
    scale = np.abs(f["sch"] * p.vcoul[igp][None, :, None]).sum(axis=(0, 1))
    assert np.all(np.abs(ach - ach_ref) <= 1e-13 * scale)
    scale = np.abs(f["ssx"] * p.vcoul[igp][None, :, None]).sum(axis=(0, 1))
    assert np.all(np.abs(asx - asx_ref) <= 1e-13 * scale)


# ---- gppsum = 1 ("half sum"), gppKerSeq.cpp ----
HALF_REF = json.loads((GOLD / "gpp_halfsum_reference.json").read_text())


def _half_closed_form(nb, nvb, nc, npg):
    """Constant fill (every complex 0.5+0.5i, vcoul 1) of the half sum.  The
    non-occupied bands contribute nothing (|wdiff|^2 >= 6.5 fails the
    inverted test); an occupied band adds, per column, (igp - 1) paired
    terms Re(s) and one unpaired s/2 with s = wtilde I_eps / (wx - wtilde)
    (and x = Omega2 / (wx^2 - wtilde^2) for asxtemp); the static remainder
    adds, per band and column, igp paired terms -2 |a|^2 Re(a) = -0.5 and the
    diagonal -|a|^2 a = -a/2, times 0.5 vcoul."""
    p = W.gpp_constant(nb, nvb, nc, npg)
    a = 0.5 + 0.5j
    wx = W.wx_frequencies()
    igp = _igp_map(p)
    igp = igp[igp >= 0]
    s = a * a / (wx - a)
    x = (a * a * a) / (wx ** 2 - a * a)
    pos = igp[igp >= 1]
    ach = nvb * 0.5 * ((pos - 1).sum() * s.real + 0.5 * len(pos) * s)
    asx = nvb * ((pos - 1).sum() * x.real + 0.5 * len(pos) * x)
    stat = nb * 0.5 * (-0.5 * igp.sum() + len(igp) * (-0.5 * a))
    return ach, asx, stat


@pytest.mark.parametrize("run", HALF_REF["runs"], ids=lambda r: "x".join(map(str, r["shape"])))
def test_halfsum_oracle_matches_reference_driver_constant_fill(run):
    """gppKerSeq.cpp run with gppsum = 1: its printed achtemp (15 digits); the
    oracle also sits on the closed form of the fill."""
    nb, nvb, nc, npg = run["shape"]
    ach, asx, _, stat = O.gpp_halfsum(W.gpp_constant(nb, nvb, nc, npg))
    ref = np.array([complex(*z) for z in run["achtemp"]])
    ex_ach, ex_asx, ex_stat = _half_closed_form(nb, nvb, nc, npg)
    if nvb == 0:
        assert np.all(ref == 0) and np.all(ach == 0)
    else:
        assert rel_err(ach, ref).max() < 1e-12
        assert rel_err(ach, ex_ach).max() < 1e-14
        assert rel_err(asx, ex_asx).max() < 1e-14
    assert abs(stat - ex_stat) <= 1e-14 * abs(ex_stat)


@pytest.mark.parametrize("name", ["half_a", "half_b", "half_c"])
def test_halfsum_oracle_matches_reference_solvers(name):
    """Per-(band, column, frequency) sch_array / ssx_array of gppKerSeq.cpp's own
    gppsum = 1 solvers (driven in its 512-wide g-vector blocks), and achstemp of
    its own reduce_achstemp, against the oracle's."""
    f = np.load(GOLD / f"gpp_halfsum_{name}.npz")
    nb, nvb, nc, ng, seed, stress = (int(x) for x in f["meta"])
    p = W.gpp_random(nb, nvb, nc, ng, seed, stress=bool(stress))
    ach, asx, n1, stat, cs, cx = O.gpp_halfsum(p, columns=True)
    assert np.abs(cs - f["sch"]).max() <= 1e-13 * np.abs(f["sch"]).max()
    assert np.abs(cx - f["ssx"]).max() <= 1e-13 * np.abs(f["ssx"]).max()
    assert abs(stat - f["achstemp"][0]) <= 1e-13 * abs(f["achstemp"][0])
    igp = _igp_map(p)
    v = p.vcoul[igp][None, :, None]
    ach_ref = (f["sch"] * v).sum(axis=(0, 1))
    assert np.all(np.abs(ach - ach_ref) <= 1e-13 * np.abs(f["sch"] * v).sum(axis=(0, 1)))
    asx_ref = (f["ssx"] * v).sum(axis=(0, 1))
    assert np.all(np.abs(asx - asx_ref) <= 1e-13 * np.abs(f["ssx"] * v).sum(axis=(0, 1)))
    assert np.abs(n1 - (f["sch"][:, :, 2] * v[:, :, 0]).sum(axis=1)).max() <= 1e-13 * np.abs(n1).max()
