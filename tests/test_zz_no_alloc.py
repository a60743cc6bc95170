"""sigma_gpp_fp64_noalloc: the GPP FP64 entry point for callers that cannot
allocate GPU memory (a framework's pool owns the device, a plug-in may not
allocate after start-up, a real-time loop cannot risk an allocation stall).

The call keeps its scratch in a fixed array inside the library.  These tests
call it through the C ABI twice in a row and compare every output with the
plan path (sigma_gpp_execute), which allocates its scratch, at the FP64 bar
of the other GPU tests: small and ragged shapes (more than one 128-band
block, so the partial slots of later band blocks are checked), a call
without acht_n1_loc, and the production shape (512 bands, 32768 g-vectors,
1638 columns; about 17 MB of the array).  The file is named to run last in
a collection.

Device memory: the array is part of the library's device image; the first
call on a device looks up its address, which may load that image (at most
the array's 32 MiB plus the image).  Every later call must leave the free
device memory exactly unchanged.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import workload as W
from conftest import rel_err
from oracle import oracle as O

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


def _check_against_plan(S, nb, nvb, nc, ng, inv, indinv, wx, d, with_n1=True):
    """Plan path once, then the no-allocation entry point twice; every output
    within the FP64 bar of the plan path, the two calls bit-identical, and
    the free device memory the same after both calls."""
    lib = S.load()
    inv = np.ascontiguousarray(inv, np.int32)
    indinv = np.ascontiguousarray(indinv, np.int32)

    # existing entry point (plan with its own scratch)
    plan = S.GppPlan(nb, nvb, nc, ng, inv, indinv, precision=S.PREC_FP64)
    ref = _outputs(nb)
    plan.execute(wx, *d, *ref)
    torch.cuda.synchronize()
    ref = _host(ref)
    plan.close()

    results = []
    free = []
    outs = [_outputs(nb) for _ in range(2)]  # allocated before the measured calls
    torch.cuda.synchronize()
    for out in outs:
        free.append(torch.cuda.mem_get_info()[0])
        st = lib.sigma_gpp_fp64_noalloc(nb, nvb, nc, ng, inv.ctypes.data, indinv.ctypes.data,
                                        wx.data_ptr(), 1.0, *[t.data_ptr() for t in d],
                                        out[0].data_ptr(), out[1].data_ptr(),
                                        out[2].data_ptr() if with_n1 else None, None)
        assert st == 0, lib.sigma_last_error_message()
        torch.cuda.synchronize()
        results.append(_host(out))
    free.append(torch.cuda.mem_get_info()[0])

    for got in results:
        assert rel_err(got[0], ref[0]).max() <= FP64_TOL
        if np.any(ref[1] != 0):
            assert rel_err(got[1], ref[1]).max() <= FP64_TOL
        if with_n1:
            assert np.abs(got[2] - ref[2]).max() <= FP64_TOL * 10 * np.abs(ref[2]).max()
        else:
            assert np.all(got[2] == 0)  # acht_n1_loc NULL: nothing written there
    # the second call reuses the scratch left by the first and gives the same bits
    for x, y in zip(results[0], results[1]):
        assert np.array_equal(x, y)
    # the first call may load the library's device image holding the array
    # (32 MiB + the image); the second takes no device memory at all
    assert free[0] - free[1] <= 40 << 20
    assert free[1] == free[2]


@pytest.mark.parametrize("case", [(96, 3, 4096, 200, 31, False), (40, 2, 1000, 37, 32, True),
                                  (300, 6, 3001, 203, 33, True)],
                         ids=["nb96-nc4096", "ragged-stress", "nb300-three-band-blocks"])
def test_noalloc_matches_plan_path_twice(sigma_lib, case):
    nb, nvb, nc, ng, seed, stress = case
    prob = W.gpp_random(nb, nvb, nc, ng, seed, stress=stress)
    d = [_dev(x) for x in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array,
                           prob.vcoul)]
    _check_against_plan(sigma_lib, nb, nvb, nc, ng, prob.inv_igp_index, prob.indinv,
                        _dev(prob.wx_array), d)


def test_noalloc_without_acht_n1_loc(sigma_lib):
    prob = W.gpp_random(150, 2, 2048, 70, 34)
    d = [_dev(x) for x in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array,
                           prob.vcoul)]
    _check_against_plan(sigma_lib, 150, 2, 2048, 70, prob.inv_igp_index, prob.indinv,
                        _dev(prob.wx_array), d, with_n1=False)


def test_noalloc_production_shape(sigma_lib):
    """512 2 32768 20 (ngpown 1638), seeded fill generated on the device."""
    S = sigma_lib
    nb, nvb, nc = 512, 2, 32768
    ng = nc // 20
    f64 = dict(dtype=torch.float64, device="cuda")
    aqsm, aqsn = torch.empty(2 * nb * nc, **f64), torch.empty(2 * nb * nc, **f64)
    ieps, wt = torch.empty(2 * ng * nc, **f64), torch.empty(2 * ng * nc, **f64)
    vcoul = torch.empty(nc, **f64)
    seed = W.GPP_PRODUCTION_SEED
    S.fill_complex_device(aqsm.data_ptr(), nb * nc, seed, W.AID_AQSM, (-1, 1), (-1, 1))
    S.fill_complex_device(aqsn.data_ptr(), nb * nc, seed, W.AID_AQSN, (-1, 1), (-1, 1))
    S.fill_complex_device(ieps.data_ptr(), ng * nc, seed, W.AID_IEPS, (-1, 1), (-1, 1))
    S.fill_complex_device(wt.data_ptr(), ng * nc, seed, W.AID_WTILDE, (0.5, 5.0), (-0.1, 0.1))
    S.fill_real_device(vcoul.data_ptr(), nc, seed, W.AID_VCOUL, 0.1, 10.0)
    inv, indinv = W.gpp_index_maps(nc, ng)
    wx = torch.tensor(W.wx_frequencies(), **f64)
    _check_against_plan(S, nb, nvb, nc, ng, inv, indinv, wx, [aqsm, aqsn, ieps, wt, vcoul])
    del aqsm, aqsn, ieps, wt
    torch.cuda.empty_cache()


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


def test_noalloc_refuses_a_capturing_stream(sigma_lib):
    """A call on a stream under graph capture returns SIGMA_ERR_UNSUPPORTED
    and queues nothing; the next plain call on the same stream succeeds."""
    S = sigma_lib
    lib = S.load()
    prob = W.gpp_random(40, 2, 1024, 40, 35)
    d = [_dev(x) for x in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array,
                           prob.vcoul)]
    wx = _dev(prob.wx_array)
    inv = np.ascontiguousarray(prob.inv_igp_index, np.int32)
    indinv = np.ascontiguousarray(prob.indinv, np.int32)
    out = _outputs(40)
    args = (40, 2, 1024, 40, inv.ctypes.data, indinv.ctypes.data, wx.data_ptr(), 1.0,
            *[t.data_ptr() for t in d], *[t.data_ptr() for t in out])
    side = torch.zeros(4, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        g.capture_begin()
        side.add_(1.0)
        st = lib.sigma_gpp_fp64_noalloc(*args, C.c_void_p(s.cuda_stream))
        g.capture_end()
    assert st == -8  # SIGMA_ERR_UNSUPPORTED
    assert b"captured" in lib.sigma_last_error_message()
    assert torch.count_nonzero(out[0]) == 0
    st = lib.sigma_gpp_fp64_noalloc(*args, C.c_void_p(s.cuda_stream))
    assert st == 0
    s.synchronize()
    ach, _, _ = O.gpp(prob)
    assert rel_err(_host(out)[0], ach).max() <= FP64_TOL
