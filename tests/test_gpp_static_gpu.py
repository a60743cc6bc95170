"""Static remainder of the GPP sum (sigma_gpp_achstemp) on the GPU against
the oracle's Fortran-formula restatement.

Bars: FP64 contraction <= 1e-12 relative on the total and on every band
(relative to the largest band); split-BF16 tensor-core contraction <= 1e-6
normwise over the bands and on the total.
"""
import numpy as np
import pytest

import workload as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
OZAKI_TOL = 1e-6

CASES = [
    # number_bands, nvband, ncouls, ngpown, seed
    (40, 2, 2048, 100, 51),
    (7, 1, 777, 33, 52),        # ragged
    (128, 2, 4096, 200, 53),
]


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "ozaki"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:4])))
def test_achstemp_matches_oracle(sigma_lib, case, mode):
    p = W.gpp_random(*case)
    ot, on1 = O.gpp_achstemp(p)
    gt, gn1 = sigma_lib.gpp_achstemp(p, mode)
    if mode == 0:
        assert abs(gt - ot) <= FP64_TOL * abs(ot)
        assert np.abs(gn1 - on1).max() <= FP64_TOL * np.abs(on1).max()
    else:
        assert abs(gt - ot) <= OZAKI_TOL * abs(ot)
        assert np.linalg.norm(gn1 - on1) <= OZAKI_TOL * np.linalg.norm(on1)


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "ozaki"])
def test_achstemp_constant_fill_and_skipped_column(sigma_lib, mode):
    c = W.gpp_constant(16, 2, 1024, 8)
    gt, gn1 = sigma_lib.gpp_achstemp(c, mode)
    exact = c.number_bands * c.ngpown * c.ncouls * (-0.125 - 0.125j)
    assert abs(gt - exact) <= (FP64_TOL if mode == 0 else OZAKI_TOL) * abs(exact)
    p = W.gpp_random(20, 2, 512, 40, 54)
    p.indinv = p.indinv.copy()
    p.indinv[p.inv_igp_index[7]] = -1            # column skipped as gppKer.cpp:328 skips it
    ot, on1 = O.gpp_achstemp(p)
    gt, gn1 = sigma_lib.gpp_achstemp(p, mode)
    tol = FP64_TOL if mode == 0 else OZAKI_TOL
    assert abs(gt - ot) <= tol * abs(ot)


def test_achstemp_index_errors(sigma_lib):
    p = W.gpp_random(4, 1, 256, 8, 55)
    p.inv_igp_index = p.inv_igp_index.copy()
    p.inv_igp_index[2] = 257
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.gpp_achstemp(p, 0)
    assert e.value.status == -2
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.gpp_achstemp(p, 7)
    assert e.value.status in (-2, -8)


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "ozaki"])
def test_static_plan_matches_host_dropin(sigma_lib, mode):
    import torch
    p = W.gpp_random(33, 2, 1500, 60, 56)
    gt, gn1 = sigma_lib.gpp_achstemp(p, mode)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.float64).copy()).cuda()
    plan = sigma_lib.StaticPlan(p.number_bands, p.ncouls, p.ngpown, p.inv_igp_index, p.indinv, mode)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    n1 = torch.zeros(2 * p.number_bands, dtype=torch.float64, device="cuda")
    vc = torch.from_numpy(p.vcoul.copy()).cuda()
    for _ in range(2):
        plan.execute(dev(p.aqsmtemp), dev(p.aqsntemp), dev(p.I_eps_array), vc, out, n1)
        torch.cuda.synchronize()
        assert plan.status() == 0
        assert out.cpu().numpy().view(np.complex128)[0] == gt
        assert np.array_equal(n1.cpu().numpy().view(np.complex128), gn1)
    plan.close()
