"""sigma_gpp_fp64_noalloc: the GPP FP64 entry point for callers that cannot
allocate GPU memory (a framework's pool owns the device, a plug-in may not
allocate after start-up, a real-time loop cannot risk an allocation stall).

The call keeps its scratch in a fixed array inside the library.  These tests
call it through the C ABI twice in a row and compare every output with the
plan path (sigma_gpp_execute), which allocates its scratch, at the FP64 bar
of the other GPU tests.  The file is named to run last in a collection.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import workload as W
from conftest import rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _dev(a):
    a = np.ascontiguousarray(a)
    if np.iscomplexobj(a):
        a = a.view(np.float64)
    return torch.from_numpy(a.copy()).cuda()


def _outputs(nb):
    return (torch.zeros(6, dtype=torch.float64, device="cuda"),
            torch.zeros(6, dtype=torch.float64, device="cuda"),
            torch.zeros(2 * nb, dtype=torch.float64, device="cuda"))


def _host(ts):
    return tuple(t.cpu().numpy().view(np.complex128).copy() for t in ts)


@pytest.mark.parametrize("case", [(96, 3, 4096, 200, 31, False), (40, 2, 1000, 37, 32, True)],
                         ids=["nb96-nc4096", "ragged-stress"])
def test_noalloc_matches_plan_path_twice(sigma_lib, case):
    nb, nvb, nc, ng, seed, stress = case
    prob = W.gpp_random(nb, nvb, nc, ng, seed, stress=stress)
    S = sigma_lib
    lib = S.load()
    d = [_dev(x) for x in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array,
                           prob.vcoul)]
    wx = _dev(prob.wx_array)
    inv = np.ascontiguousarray(prob.inv_igp_index, np.int32)
    indinv = np.ascontiguousarray(prob.indinv, np.int32)

    # existing entry point (plan with its own scratch)
    plan = S.GppPlan(nb, nvb, nc, ng, inv, indinv, precision=S.PREC_FP64)
    ref = _outputs(nb)
    plan.execute(wx, *d, *ref)
    torch.cuda.synchronize()
    ref = _host(ref)
    plan.close()

    results = []
    free_after = []
    for _ in range(2):
        out = _outputs(nb)
        st = lib.sigma_gpp_fp64_noalloc(nb, nvb, nc, ng, inv.ctypes.data, indinv.ctypes.data,
                                        wx.data_ptr(), 1.0, *[t.data_ptr() for t in d],
                                        *[t.data_ptr() for t in out], None)
        assert st == 0, lib.sigma_last_error_message()
        torch.cuda.synchronize()
        free_after.append(torch.cuda.mem_get_info()[0])
        results.append(_host(out))

    for got in results:
        assert rel_err(got[0], ref[0]).max() <= FP64_TOL
        if np.any(ref[1] != 0):
            assert rel_err(got[1], ref[1]).max() <= FP64_TOL
        assert np.abs(got[2] - ref[2]).max() <= FP64_TOL * 10 * np.abs(ref[2]).max()
    # the second call reuses the scratch left by the first and gives the same bits
    for x, y in zip(results[0], results[1]):
        assert np.array_equal(x, y)
    # no device memory was taken between the two calls
    assert free_after[0] == free_after[1]


def test_noalloc_rejects_problems_beyond_its_scratch(sigma_lib):
    lib = sigma_lib.load()
    ng = 70000  # more columns than the static column map holds
    nc = ng
    inv = np.arange(1, ng + 1, dtype=np.int32)
    indinv = np.arange(nc, dtype=np.int32)
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = dummy.data_ptr()
    st = lib.sigma_gpp_fp64_noalloc(4, 1, nc, ng, inv.ctypes.data, indinv.ctypes.data, p, 1.0,
                                    p, p, p, p, p, p, p, p, None)
    assert st == -9  # SIGMA_ERR_WORKSPACE
    assert b"65536" in lib.sigma_last_error_message()
    # too many partial sums for the 32 MiB array: a very tall band count
    ng, nc, nb = 4096, 8192, 60000
    inv = ((np.arange(ng) + 1) * nc // ng).astype(np.int32)
    indinv = np.arange(nc, dtype=np.int32)
    st = lib.sigma_gpp_fp64_noalloc(nb, 1, nc, ng, inv.ctypes.data, indinv.ctypes.data, p, 1.0,
                                    p, p, p, p, p, p, p, p, None)
    assert st == -9
    assert b"32 MiB" in lib.sigma_last_error_message()
