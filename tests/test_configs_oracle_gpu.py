"""Every output of the production workloads against the CPU oracle.

The oracle's full outputs of each workload are committed fixtures
(tests/golden/make_config_fixtures.py: oracle/gpp_oracle.cpp, the
compensated restatement of BGW-Kernels/gppKer.cpp:19-65,130-159,387-439,
pinned to the unmodified reference by test_oracle.py).  The GPU side
regenerates the same seeded inputs on the device (bit-identical to the host
generator, test_gpp_gpu.py::test_device_fill_matches_host_generator).

Bars, on every achtemp[iw] / asxtemp[iw]:
  FP64 form                 <= 1e-12 relative
  mixed and tensor forms    <= 1e-6 relative (plain, no error model)
acht_n1_loc: FP64 per band <= 1e-12 relative (bands whose value is at least
1e-3 of the largest; the others <= 1e-15 of the largest in absolute terms),
the mixed and tensor forms <= 1e-6 normwise.  FF schDt: FP64 <= 1e-12 per
entry, split-BF16 form <= 1e-6 normwise.

Workloads: 512 bands, nvband 2, ncouls 32768, nodes_per_group 20 (ngpown
1638), seed 1; the same with 5 % of wtilde within 1e-3 of a frequency,
seed 2; the 48 uneven instances of workload.batched_shapes(); FF 512 bands,
ncouls 16384, ngpown 820, nfreq 15, seed 4.
"""
import pathlib

import numpy as np
import pytest
import torch

import workload as W
from conftest import normwise_err

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
FP64_TOL = 1e-12
MIXED_TOL = 1e-6
FORMS = [(0, "fp64", FP64_TOL), (1, "mixed", MIXED_TOL), (2, "tensor", MIXED_TOL)]


def _fixture(name):
    with np.load(GOLDEN / name) as z:
        return {k: z[k] for k in z.files}


def _rel(a, b):
    return np.abs(a - b) / np.abs(b)


def _check(out, ref, tol, name):
    ach, asx, n1 = out
    e_ach, e_asx = _rel(ach, ref["achtemp"]), _rel(asx, ref["asxtemp"])
    assert e_ach.max() <= tol, (name, "achtemp", e_ach)
    assert e_asx.max() <= tol, (name, "asxtemp", e_asx)
    on1 = ref["acht_n1_loc"]
    if tol == FP64_TOL:
        scale = np.abs(on1).max()
        big = np.abs(on1) >= 1e-3 * scale
        assert _rel(n1[big], on1[big]).max() <= FP64_TOL, name
        assert np.abs(n1[~big] - on1[~big]).max(initial=0.0) <= 1e-15 * scale, name
    else:
        assert normwise_err(n1, on1) <= MIXED_TOL, name


class DeviceInstance:
    def __init__(self, S, nb, nvb, nc, ng, seed, stress=False):
        f64 = dict(dtype=torch.float64, device="cuda")
        self.S, self.nb, self.nvb, self.nc, self.ng = S, nb, nvb, nc, ng
        self.aqsm = torch.empty(2 * nb * nc, **f64)
        self.aqsn = torch.empty_like(self.aqsm)
        self.ieps = torch.empty(2 * ng * nc, **f64)
        self.wt = torch.empty_like(self.ieps)
        self.vcoul = torch.empty(nc, **f64)
        S.fill_complex_device(self.aqsm.data_ptr(), nb * nc, seed, W.AID_AQSM, (-1, 1), (-1, 1))
        S.fill_complex_device(self.aqsn.data_ptr(), nb * nc, seed, W.AID_AQSN, (-1, 1), (-1, 1))
        S.fill_complex_device(self.ieps.data_ptr(), ng * nc, seed, W.AID_IEPS, (-1, 1), (-1, 1))
        S.fill_complex_device(self.wt.data_ptr(), ng * nc, seed, W.AID_WTILDE, (0.5, 5.0), (-0.1, 0.1))
        if stress:
            S.fill_stress_device(self.wt.data_ptr(), ng * nc, seed, W.AID_STRESS, W.wx_frequencies())
        S.fill_real_device(self.vcoul.data_ptr(), nc, seed, W.AID_VCOUL, 0.1, 10.0)
        self.inv, self.indinv = W.gpp_index_maps(nc, ng)
        self.wx = torch.tensor(W.wx_frequencies(), **f64)

    def run(self, prec):
        plan = self.S.GppPlan(self.nb, self.nvb, self.nc, self.ng, self.inv, self.indinv, precision=prec)
        f64 = dict(dtype=torch.float64, device="cuda")
        ach, asx, n1 = torch.zeros(6, **f64), torch.zeros(6, **f64), torch.zeros(2 * self.nb, **f64)
        plan.execute(self.wx, self.aqsm, self.aqsn, self.ieps, self.wt, self.vcoul, ach, asx, n1)
        torch.cuda.synchronize()
        assert plan.status() == 0
        plan.close()
        return tuple(t.cpu().numpy().view(np.complex128).copy() for t in (ach, asx, n1))


@pytest.mark.parametrize("fixture,stress", [("config_gpp_production.npz", False),
                                            ("config_gpp_stress.npz", True)], ids=["production", "stress"])
def test_production_every_output_vs_oracle(sigma_lib, fixture, stress):
    ref = _fixture(fixture)
    nb, nvb, nc, ng, seed, st = (int(x) for x in ref["meta"])
    assert bool(st) == stress
    inst = DeviceInstance(sigma_lib, nb, nvb, nc, ng, seed, stress=stress)
    for prec, name, tol in FORMS:
        _check(inst.run(prec), ref, tol, f"{fixture}:{name}")
    del inst
    torch.cuda.empty_cache()


@pytest.fixture(scope="module")
def batch48(sigma_lib):
    import batched
    xs = batched.device_instances()
    yield xs
    del xs
    torch.cuda.empty_cache()


@pytest.mark.parametrize("prec,name,tol", FORMS, ids=[f[1] for f in FORMS])
def test_batch48_every_output_vs_oracle(sigma_lib, batch48, prec, name, tol):
    ref = _fixture("config_gpp_batched.npz")
    xs = batch48
    assert len(xs) == len(ref["meta"])
    b = sigma_lib.GppBatch([x.as_dict() for x in xs], precision=prec)
    s = torch.cuda.Stream()
    b.launch_graph(s.cuda_stream)
    s.synchronize()
    assert b.status(s.cuda_stream) == 0
    off = ref["n1_offsets"]
    for i, x in enumerate(xs):
        assert [x.nb, x.nvb, x.nc, x.ng, x.seed] == [int(v) for v in ref["meta"][i]]
        r = {"achtemp": ref["achtemp"][i], "asxtemp": ref["asxtemp"][i],
             "acht_n1_loc": ref["acht_n1_loc"][off[i]:off[i + 1]]}
        _check(x.outputs(), r, tol, f"instance {i}:{name}")
    b.close()


def test_ff_production_every_entry_vs_oracle(sigma_lib):
    ref = _fixture("config_ff_schdt.npz")
    nb, nc, ng, nf, seed = (int(x) for x in ref["meta"])
    f64 = dict(dtype=torch.float64, device="cuda")
    S = sigma_lib
    epsr = torch.empty(2 * nf * ng * nc, **f64)
    aqsn = torch.empty(2 * nb * nc, **f64)
    aqsm = torch.empty_like(aqsn)
    S.fill_complex_device(epsr.data_ptr(), nf * ng * nc, seed, W.AID_IEPSR, (-1, 1), (-1, 1))
    S.fill_complex_device(aqsn.data_ptr(), nb * nc, seed, W.AID_AQSN, (-1, 1), (-1, 1))
    S.fill_complex_device(aqsm.data_ptr(), nb * nc, seed, W.AID_AQSM, (-1, 1), (-1, 1))
    inv, indinv = W.ff_index_maps(nc, ng)
    o = ref["schdt"]
    for mode in (0, 1):
        plan = S.FfPlan(nb, nc, ng, nf, inv, indinv, mode)
        out = torch.zeros(2 * nb * nf, **f64)
        plan.execute(epsr, aqsn, aqsm, out)
        torch.cuda.synchronize()
        assert plan.status() == 0
        plan.close()
        g = out.cpu().numpy().view(np.complex128).reshape(nb, nf)
        if mode == 0:
            assert _rel(g, o).max() <= FP64_TOL
        else:
            assert normwise_err(g, o) <= MIXED_TOL
    del epsr, aqsn, aqsm
    torch.cuda.empty_cache()
