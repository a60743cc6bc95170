"""FF schDt contraction on the GPU through the C ABI, against the CPU oracle.

Bars: the FP64 form <= 1e-12 relative to max|schDt| on every entry; the
split-BF16 tensor-core form <= 1e-6 normwise (||G - O|| / ||O||) and
<= 1e-6 on every entry relative to max|schDt|.
"""
import numpy as np
import pytest
import torch

import workload as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
OZAKI_TOL = 1e-6


def _errs(g, o):
    scale = np.abs(o).max()
    return np.abs(g - o).max() / scale, np.linalg.norm(g - o) / np.linalg.norm(o)


CASES = [
    # number_bands, ncouls, ngpown, nfreq, seed
    (70, 1000, 70, 3, 5),      # ragged: nothing a multiple of the tiles
    (128, 4096, 200, 4, 6),
    (33, 257, 129, 2, 7),
    (64, 640, 64, 5, 8),       # exact multiples
    (1, 64, 20, 1, 9),         # one band, one frequency
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:4])))
def test_ff_fp64_matches_oracle(sigma_lib, case):
    p = W.ff_random(*case)
    o = O.ff_schdt(p).reshape(p.number_bands, p.nfreq)
    g = sigma_lib.ff_host(p, sigma_lib.FF_MODE_FP64)
    assert _errs(g, o)[0] <= FP64_TOL


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:4])))
def test_ff_ozaki_matches_oracle(sigma_lib, case):
    p = W.ff_random(*case)
    o = O.ff_schdt(p).reshape(p.number_bands, p.nfreq)
    g = sigma_lib.ff_host(p, sigma_lib.FF_MODE_OZAKI_BF16)
    emax, enorm = _errs(g, o)
    assert enorm <= OZAKI_TOL and emax <= OZAKI_TOL


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "ozaki"])
def test_ff_constant_fill_closed_form(sigma_lib, mode):
    # FFKer_cori/ffKernel.cpp fill (:398-433): every complex 0.5+0.5i, inv_igp_index[i] = i
    c = W.ff_constant(6, 300, 40, 3)
    g = sigma_lib.ff_host(c, mode)
    exact = 40 * 300 * 0.5 * (0.5 + 0.5j)
    assert np.abs(g - exact).max() / abs(exact) <= (FP64_TOL if mode == 0 else OZAKI_TOL)


def test_ff_index_errors(sigma_lib):
    p = W.ff_random(4, 128, 20, 2, 3)
    p.inv_igp_index = p.inv_igp_index.copy()
    p.inv_igp_index[3] = 128  # indinv read out of bounds
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.ff_host(p, 0)
    assert e.value.status == -2
    p = W.ff_random(4, 16, 20, 2, 3)  # ngpown > ncouls, rejected as ffKernel.cpp:320-325 does
    with pytest.raises(sigma_lib.SigmaError) as e:
        sigma_lib.ff_host(p, 0)
    assert e.value.status == -1


class FFProduction:
    """number_bands 512, ncouls 16384, ngpown 820, nfreq 15, seeded on the device."""

    def __init__(self, S):
        nb, nc, ng, nf = 512, 16384, 820, 15
        self.shape = (nb, nc, ng, nf)
        self.epsr = torch.empty(2 * nf * ng * nc, dtype=torch.float64, device="cuda")
        self.aqsn = torch.empty(2 * nb * nc, dtype=torch.float64, device="cuda")
        self.aqsm = torch.empty_like(self.aqsn)
        S.fill_complex_device(self.epsr.data_ptr(), nf * ng * nc, W.FF_SEED, W.AID_IEPSR, (-1, 1), (-1, 1))
        S.fill_complex_device(self.aqsn.data_ptr(), nb * nc, W.FF_SEED, W.AID_AQSN, (-1, 1), (-1, 1))
        S.fill_complex_device(self.aqsm.data_ptr(), nb * nc, W.FF_SEED, W.AID_AQSM, (-1, 1), (-1, 1))
        self.inv, self.indinv = W.ff_index_maps(nc, ng)
        self.S = S

    def run(self, mode, reps=1):
        nb, nc, ng, nf = self.shape
        plan = self.S.FfPlan(nb, nc, ng, nf, self.inv, self.indinv, mode)
        outs = []
        for _ in range(reps):
            out = torch.zeros(2 * nb * nf, dtype=torch.float64, device="cuda")
            plan.execute(self.epsr, self.aqsn, self.aqsm, out)
            torch.cuda.synchronize()
            assert plan.status() == 0
            outs.append(out.cpu().numpy().view(np.complex128).reshape(nb, nf))
        plan.close()
        return outs

    def host(self):
        nb, nc, ng, nf = self.shape
        v = lambda t: t.cpu().numpy().view(np.complex128)
        return W.FFProblem(nb, nc, ng, nf, self.inv, self.indinv, v(self.epsr).reshape(nf, ng, nc),
                           v(self.aqsn).reshape(nb, nc), v(self.aqsm).reshape(nb, nc))


@pytest.fixture(scope="module")
def ffprod(sigma_lib):
    p = FFProduction(sigma_lib)
    yield p
    del p
    torch.cuda.empty_cache()


def test_ff_production_sampled_entries(ffprod):
    g64 = ffprod.run(0)[0]
    goz = ffprod.run(1)[0]
    entries = [(0, 0), (511, 14), (100, 7), (300, 3), (257, 11), (63, 1)]
    o = O.ff_schdt(ffprod.host(), entries)
    scale = np.abs(g64).max()
    for (n, f), v in zip(entries, o):
        assert abs(g64[n, f] - v) <= FP64_TOL * scale
        assert abs(goz[n, f] - v) <= OZAKI_TOL * scale
    assert np.linalg.norm(goz - g64) / np.linalg.norm(g64) <= OZAKI_TOL


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "ozaki"])
def test_ff_production_repeatable_and_linear(ffprod, mode):
    a, b = ffprod.run(mode, reps=2)
    assert np.array_equal(a, b)
    # schDt is linear in aqsm (conj): doubling aqsm doubles it exactly
    keep = ffprod.aqsm.clone()
    ffprod.aqsm.mul_(2.0)
    try:
        c = ffprod.run(mode)[0]
    finally:
        ffprod.aqsm.copy_(keep)
    assert np.array_equal(2.0 * a, c)
