"""Failure detection on the GPU without a GPU fault.

Every spin-wait in the kernels is bounded and records SIGMA_ERR_TIMEOUT in
the launch's status word instead of hanging.  Here a wait is made to run out
the allowed way: the FP64 shared-frequency main pass runs gated on words
that nothing ever writes (sigma_gpp_selftest_gate_timeout), with a short
bound.  The call must come back promptly with SIGMA_ERR_TIMEOUT, the CUDA
context must stay usable, and the next execution must start from a cleared
status and give the same bits as before.  (The reference has no device
waits; it checks its arguments only, BGW-Kernels/gppKer.cpp:164-169.)
"""
import time

import numpy as np
import pytest
import torch

import workload as W
from conftest import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SIGMA_ERR_TIMEOUT = -5


def _dev(a):
    a = np.ascontiguousarray(a)
    if np.iscomplexobj(a):
        a = a.view(np.float64)
    return torch.from_numpy(a.copy()).cuda()


def _execute(plan, wx, d, nb):
    ach = torch.zeros(6, dtype=torch.float64, device="cuda")
    asx = torch.zeros_like(ach)
    n1 = torch.zeros(2 * nb, dtype=torch.float64, device="cuda")
    plan.execute(wx, *d, ach, asx, n1)
    torch.cuda.synchronize()
    return tuple(t.cpu().numpy().view(np.complex128).copy() for t in (ach, asx, n1))


def test_gate_wait_times_out_and_the_next_call_succeeds(sigma_lib):
    prob = W.gpp_random(150, 2, 4096, 120, 41)  # two 128-band blocks, several column blocks
    plan = sigma_lib.GppPlan(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, prob.inv_igp_index,
                             prob.indinv, precision=sigma_lib.PREC_FP64)
    d = [_dev(x) for x in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array, prob.vcoul)]
    wx = _dev(prob.wx_array)
    before = _execute(plan, wx, d, prob.number_bands)
    assert plan.status() == 0

    # gate words nothing writes, each wait bounded by 4000 polls 256 ns apart
    t0 = time.perf_counter()
    st = plan.selftest_gate_timeout(wx, *d, wait_polls=4000)
    dt = time.perf_counter() - t0
    assert st == SIGMA_ERR_TIMEOUT
    assert dt < 5.0  # the kernel dropped its items after the first wait gave up
    assert plan.status() == SIGMA_ERR_TIMEOUT  # status kept until the next execution
    torch.cuda.synchronize()  # the context is still usable

    after = _execute(plan, wx, d, prob.number_bands)
    assert plan.status() == 0
    for x, y in zip(before, after):
        assert np.array_equal(x, y)
    ach, asx, _ = O.gpp(prob)
    assert rel_err(after[0], ach).max() <= 1e-12
    assert rel_err(after[1], asx).max() <= 1e-12

    # the host drop-in on the same device also starts from a clean state
    g = sigma_lib.gpp_host(prob, sigma_lib.PREC_FP64)
    assert rel_err(g[0], ach).max() <= 1e-12
    plan.close()


def test_gate_selftest_refuses_other_plans(sigma_lib):
    prob = W.gpp_random(40, 2, 1024, 40, 42)
    plan = sigma_lib.GppPlan(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, prob.inv_igp_index,
                             prob.indinv, precision=sigma_lib.PREC_MIXED)
    d = [_dev(x) for x in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array, prob.vcoul)]
    wx = _dev(prob.wx_array)
    assert plan.selftest_gate_timeout(wx, *d, wait_polls=100) == -8  # SIGMA_ERR_UNSUPPORTED
    plan.close()
