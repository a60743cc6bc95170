"""Device-resident GPP instances for the batched path.

A sigma calculation evaluates many (q-point, band window) GPP instances of
uneven shape; `workload.batched_shapes()` draws a seeded set of 48 of them.
`DeviceInstance` fills one instance on the GPU with the seeded generator
(bit-identical to `workload.fill_*` on the host) and holds its output arrays;
`as_dict()` is the sigma_gpp_instance the batch API takes.
"""
from __future__ import annotations

import numpy as np
import torch

import sigma_gb300 as S
import workload as W


class DeviceInstance:
    def __init__(self, number_bands, nvband, ncouls, ngpown, seed, stress=False, per_band_wx=False, **_):
        nb, nc, ng = number_bands, ncouls, ngpown
        self.nb, self.nvb, self.nc, self.ng, self.seed = nb, nvband, nc, ng, seed
        f64 = dict(dtype=torch.float64, device="cuda")
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
        # per_band_wx: the same three frequencies stored once per band
        # (wx_array[n1][3], stride 3), which selects the per-band kernels
        wx = W.wx_frequencies()
        self.wx_stride = 3 if per_band_wx else 0
        self.wx = torch.tensor(np.tile(wx, nb) if per_band_wx else wx, **f64)
        self.ach = torch.zeros(6, **f64)
        self.asx = torch.zeros(6, **f64)
        self.n1 = torch.zeros(2 * nb, **f64)

    @property
    def terms(self) -> int:
        return self.nb * self.ng * self.nc * 3

    @property
    def input_bytes(self) -> int:
        return 8 * (self.aqsm.numel() + self.aqsn.numel() + self.ieps.numel() + self.wt.numel()
                    + self.vcoul.numel())

    def as_dict(self):
        return dict(number_bands=self.nb, nvband=self.nvb, ncouls=self.nc, ngpown=self.ng,
                    inv_igp_index=self.inv, indinv=self.indinv, wx_array=self.wx,
                    wx_band_stride=self.wx_stride,
                    occ=1.0, aqsmtemp=self.aqsm, aqsntemp=self.aqsn, I_eps_array=self.ieps,
                    wtilde_array=self.wt, vcoul=self.vcoul, achtemp=self.ach, asxtemp=self.asx,
                    acht_n1_loc=self.n1)

    def outputs(self):
        """(achtemp[3], asxtemp[3], acht_n1_loc[nb]) as complex128 host arrays."""
        return tuple(t.cpu().numpy().view(np.complex128).copy() for t in (self.ach, self.asx, self.n1))

    def run_single(self, precision):
        """The same instance through a single-instance plan; returns its outputs."""
        plan = S.GppPlan(self.nb, self.nvb, self.nc, self.ng, self.inv, self.indinv, precision=precision)
        f64 = dict(dtype=torch.float64, device="cuda")
        ach, asx, n1 = torch.zeros(6, **f64), torch.zeros(6, **f64), torch.zeros(2 * self.nb, **f64)
        plan.execute(self.wx, self.aqsm, self.aqsn, self.ieps, self.wt, self.vcoul, ach, asx, n1,
                     wx_band_stride=self.wx_stride)
        torch.cuda.synchronize()
        plan.close()
        return tuple(t.cpu().numpy().view(np.complex128) for t in (ach, asx, n1))

    def host_problem(self) -> W.GppProblem:
        c = lambda t, r: t.cpu().numpy().view(np.complex128).reshape(r, self.nc)
        return W.GppProblem(self.nb, self.nvb, self.nc, self.ng, self.inv, self.indinv,
                            W.wx_frequencies(), c(self.aqsm, self.nb), c(self.aqsn, self.nb),
                            c(self.ieps, self.ng), c(self.wt, self.ng), self.vcoul.cpu().numpy())


def device_instances(shapes=None):
    """DeviceInstance for every shape (default: the 48 seeded batched shapes)."""
    return [DeviceInstance(**s) for s in (shapes if shapes is not None else W.batched_shapes())]
