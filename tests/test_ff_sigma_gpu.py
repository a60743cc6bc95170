"""Full-frequency sigma (sigma_ff_sigma) on the GPU against the oracle's
restatement of the Fortran band loop (itself pinned to the reference's
FFKer_cori kernels in tests/test_oracle.py).

Bars: contractions in FP64 -> every output within 1e-12 of the oracle,
relative to the largest magnitude of that output array; split-BF16
tensor-core contractions -> within 1e-6 normwise per output array and on
achsDtemp.
"""
import numpy as np
import pytest

import workload as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
OZAKI_TOL = 1e-6
KEYS = ("asxDtemp", "achDtemp", "achDtemp_cor", "achDtemp_corb", "ach2Dtemp")

CASES = [
    # number_bands, nvband, ncouls, ngpown, nfreq, nfreqeval, seed, freqevalmin
    (12, 2, 300, 20, 8, 4, 7, 0.3),
    (30, 4, 777, 33, 10, 6, 9, 0.0),      # wx on grid points, some wx < 0
    (16, 16, 512, 40, 6, 5, 11, 2.0),     # every band occupied
    (20, 0, 256, 24, 12, 3, 12, 1.25),    # no occupied band
]


def _cmp(g, o, tol, normwise):
    a, b = complex(g["achsDtemp"]), complex(o["achsDtemp"])
    assert abs(a - b) <= tol * abs(b)
    for k in KEYS:
        x, y = g[k], o[k]
        scale = np.abs(y).max()
        if scale == 0:
            assert np.abs(x).max() <= tol
            continue
        if normwise:
            assert np.linalg.norm(x - y) <= tol * np.linalg.norm(y), k
        else:
            assert np.abs(x - y).max() <= tol * scale, k


def _prob(case):
    nb, nv, nc, ng, nf, ne, seed, fmin = case
    p = W.ff_sigma_random(nb, nv, nc, ng, nf, ne, seed)
    p.freqevalmin = fmin
    return p


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "ozaki"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:6])))
def test_ff_sigma_matches_oracle_zero_schdt(sigma_lib, case, mode):
    p = _prob(case)
    o = O.ff_sigma(p)
    g = sigma_lib.ff_sigma(p, mode, schdt="zero")
    _cmp(g, o, FP64_TOL if mode == 0 else OZAKI_TOL, mode == 1)


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "ozaki"])
@pytest.mark.parametrize("case", CASES[:2], ids=lambda c: "x".join(map(str, c[:6])))
def test_ff_sigma_with_computed_schdt(sigma_lib, case, mode):
    """schDt_matrix NULL: the library contracts I_epsR itself (the Fortran's
    commented zgemm); the oracle gets the oracle's own schDt."""
    p = _prob(case)
    sd = O.ff_schdt(p.ff_problem()).reshape(p.number_bands, p.nfreq)
    o = O.ff_sigma(p, sd)
    g = sigma_lib.ff_sigma(p, mode, schdt="compute")
    _cmp(g, o, FP64_TOL if mode == 0 else OZAKI_TOL, mode == 1)
    # the same with schDt passed in explicitly
    g2 = sigma_lib.ff_sigma(p, mode, schdt=sd)
    _cmp(g2, o, FP64_TOL if mode == 0 else OZAKI_TOL, mode == 1)


def test_ff_sigma_constant_fill_matches_reference_driver(sigma_lib):
    import json
    import pathlib
    ref = json.loads((pathlib.Path(__file__).parent / "golden" / "ff_sigma_reference.json").read_text())
    for run in ref["constant_fill"]:
        p = W.ff_sigma_constant(*run["shape"])
        g = sigma_lib.ff_sigma(p, 0, schdt="zero")
        for key, ours in (("achsDtemp", g["achsDtemp"]), ("asxDtemp", g["asxDtemp"][0]),
                          ("achDtemp_cor", g["achDtemp_cor"][0])):
            r = complex(*run[key])
            assert abs(ours - r) <= 1e-6 + 1e-12 * abs(r)


def test_ff_sigma_argument_errors(sigma_lib):
    p = _prob(CASES[0])
    q = W.FFSigmaProblem(**p.__dict__)
    q.inv_igp_index = p.inv_igp_index.copy()
    q.inv_igp_index[3] = p.ncouls          # indinv read out of bounds
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.ff_sigma(q, 0)
    assert e.value.status == -2
    q = W.FFSigmaProblem(**p.__dict__)
    q.dFreqGrid = p.dFreqGrid[::-1].copy()  # descending grid
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.ff_sigma(q, 0)
    assert e.value.status == -1


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "ozaki"])
def test_ff_sigma_plan_matches_host_dropin(sigma_lib, mode):
    import torch
    p = _prob(CASES[1])
    g = sigma_lib.ff_sigma(p, mode, schdt="compute")
    dc = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128).view(np.float64).copy()).cuda()
    df = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).copy()).cuda()
    plan = sigma_lib.FfSigmaPlan(p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nfreq, p.nfreqeval,
                                 p.inv_igp_index, p.indinv, mode)
    out = torch.zeros(2 * (1 + 5 * p.nfreqeval), dtype=torch.float64, device="cuda")
    args = [dc(p.aqsmtemp), dc(p.aqsntemp), dc(p.I_epsR), dc(p.I_epsA), df(p.vcoul), df(p.ekq),
            df(p.dFreqGrid), dc(p.dFreqBrd), df(p.pref)]
    for _ in range(2):
        plan.execute(*args, p.pref_zb, p.freqevalmin, p.freqevalstep, p.occ, None, out)
        torch.cuda.synchronize()
        assert plan.status() == 0
        r = sigma_lib.FfSigmaPlan.unpack(out.cpu().numpy(), p.nfreqeval)
        assert r["achsDtemp"] == g["achsDtemp"]
        for k in KEYS:
            assert np.array_equal(r[k], g[k])
    plan.close()
