"""Real-valued GPP (sigma_gpp_real_fp64) on the GPU against the oracle's
restatement of gppKer_real.cpp (pinned to the reference's own driver and
occupied-band solver in tests/test_oracle.py).

Bar: every achtemp / asxtemp output within 1e-12 relative of the oracle
(1e-12 of the sum of |terms| for an output whose terms cancel to zero);
acht_n1_loc within 1e-12 of its largest entry.
"""
import json
import pathlib

import numpy as np
import pytest

import workload as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-12

CASES = [
    # number_bands, nvband, ncouls, ngpown, seed
    (40, 3, 2048, 100, 61),
    (33, 1, 1000, 37, 62),        # ragged
    (7, 0, 333, 5, 63),           # no occupied band
    (9, 9, 777, 21, 64),          # every band occupied
    (130, 2, 4096, 70, 65),       # several 64-band blocks
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:4])))
def test_real_matches_oracle(sigma_lib, case):
    p = W.gpp_real_random(*case)
    o = O.gpp_real(p)
    g = sigma_lib.gpp_real_host(p)
    assert np.all(np.abs(g[0] - o[0]) <= TOL * np.abs(o[0]))
    if np.any(o[1] != 0):
        assert np.all(np.abs(g[1] - o[1]) <= TOL * np.maximum(np.abs(o[1]), 1e-3 * np.abs(o[1]).max()))
    else:
        assert np.all(g[1] == 0)
    assert np.abs(g[2] - o[2]).max() <= TOL * 10 * np.abs(o[2]).max()


def test_real_constant_fill_matches_reference_driver(sigma_lib):
    ref = json.loads((pathlib.Path(__file__).parent / "golden" / "gpp_real_reference.json").read_text())
    for run in ref["runs"]:
        g = sigma_lib.gpp_real_host(W.gpp_real_constant(*run["shape"]))
        r = np.array(run["achtemp"])
        assert np.abs(g[0] - r).max() <= 1e-12 * np.abs(r).max()


def test_real_exact_pole_and_skipped_column(sigma_lib):
    p = W.gpp_real_random(12, 2, 512, 20, 66)
    p.wtilde_array = p.wtilde_array.copy()
    p.wtilde_array[3, 7] = p.wx_array[1]           # wx - wtilde = 0: dropped, never divided
    p.indinv = p.indinv.copy()
    p.indinv[p.inv_igp_index[5]] = -1               # column skipped as gppKer_real.cpp:321 skips it
    o = O.gpp_real(p)
    g = sigma_lib.gpp_real_host(p)
    assert np.all(np.isfinite(g[0])) and np.all(np.isfinite(g[1]))
    assert np.all(np.abs(g[0] - o[0]) <= TOL * np.abs(o[0]))


def test_real_plan_repeatable(sigma_lib):
    import torch
    p = W.gpp_real_random(70, 2, 3000, 75, 67)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).copy()).cuda()
    plan = sigma_lib.GppRealPlan(p.number_bands, p.nvband, p.ncouls, p.ngpown, p.inv_igp_index, p.indinv)
    args = [d(p.wx_array), d(p.aqsmtemp), d(p.aqsntemp), d(p.I_eps_array), d(p.wtilde_array), d(p.vcoul)]
    outs = []
    for _ in range(2):
        ach, asx, n1 = (torch.zeros(3, dtype=torch.float64, device="cuda"),
                        torch.zeros(3, dtype=torch.float64, device="cuda"),
                        torch.zeros(p.number_bands, dtype=torch.float64, device="cuda"))
        plan.execute(*args, ach, asx, n1)
        torch.cuda.synchronize()
        outs.append([t.cpu().numpy() for t in (ach, asx, n1)])
    plan.close()
    for x, y in zip(*outs):
        assert np.array_equal(x, y)
    h = sigma_lib.gpp_real_host(p)
    for x, y in zip(outs[0], h):
        assert np.array_equal(x, y)
