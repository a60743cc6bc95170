"""Full-output oracle fixtures of the production workloads (CPU, once).

The oracle (oracle/gpp_oracle.cpp: compensated restatement of
BGW-Kernels/gppKer.cpp:19-65,130-159,387-439, pinned to the unmodified
reference by tests/test_oracle.py) evaluates every output of each workload
below on the seeded inputs that fortkernels-_gb300/workload.py (host) and
csrc/tools.cu (device, bit-identical) generate.  The GPU tests regenerate the
same inputs on the device and compare every output with these files, so the
production-size parity checks need no CPU oracle run at test time.

  config_gpp_production.npz  512 bands, nvband 2, ncouls 32768, ngpown 1638,
                             seed 1: achtemp[3], asxtemp[3], acht_n1_loc[512],
                             and sum |term|^2 per achtemp / asxtemp output
  config_gpp_stress.npz      the same shape, seed 2, 5 % of wtilde within 1e-3
                             of a frequency
  config_gpp_batched.npz     the 48 instances of workload.batched_shapes()
                             (seeds 1000 + i): shapes, achtemp, asxtemp,
                             acht_n1_loc (concatenated, offsets), sum |term|^2
  config_ff_schdt.npz        FF schDt[512][15] (ncouls 16384, ngpown 820,
                             seed 4; ffkernel.deslippe.best.f90:402-418 in the
                             C layouts of FFKer_cori/ffKernel.cpp)

Run:  python tests/golden/make_config_fixtures.py [production] [stress] [ff] [batched]
(about 70 minutes on 8 cores for all four).
"""
from __future__ import annotations

import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "fortkernels-_gb300"))
sys.path.insert(0, str(ROOT))

import workload as W  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _gpp_outputs(prob):
    ach, asx, n1 = O.gpp(prob)
    a2, x2 = O.gpp_abs2(prob)
    return ach, asx, n1, a2, x2


def production(stress=False):
    seed = W.GPP_STRESS_SEED if stress else W.GPP_PRODUCTION_SEED
    s = W.GPP_PRODUCTION
    prob = W.gpp_random(s["number_bands"], s["nvband"], s["ncouls"], 0, seed, stress=stress,
                        nodes_per_group=s["nodes_per_group"])
    ach, asx, n1, a2, x2 = _gpp_outputs(prob)
    name = "config_gpp_stress.npz" if stress else "config_gpp_production.npz"
    np.savez_compressed(HERE / name, achtemp=ach, asxtemp=asx, acht_n1_loc=n1, achtemp_abs2=a2,
                        asxtemp_abs2=x2,
                        meta=np.array([prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, seed,
                                       int(stress)]))
    print(name, ach, asx, flush=True)


def batched():
    shapes = W.batched_shapes()
    meta, ach, asx, a2, x2, n1, off = [], [], [], [], [], [], [0]
    for i, s in enumerate(shapes):
        t0 = time.time()
        prob = W.gpp_random(s["number_bands"], s["nvband"], s["ncouls"], s["ngpown"], s["seed"])
        a, x, n, aa, xx = _gpp_outputs(prob)
        meta.append([s["number_bands"], s["nvband"], s["ncouls"], s["ngpown"], s["seed"]])
        ach.append(a)
        asx.append(x)
        a2.append(aa)
        x2.append(xx)
        n1.append(n)
        off.append(off[-1] + len(n))
        print(f"instance {i}: {s} {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(HERE / "config_gpp_batched.npz", meta=np.array(meta), achtemp=np.array(ach),
                        asxtemp=np.array(asx), achtemp_abs2=np.array(a2), asxtemp_abs2=np.array(x2),
                        acht_n1_loc=np.concatenate(n1), n1_offsets=np.array(off))


def ff():
    s = W.FF_PRODUCTION
    prob = W.ff_random(s["number_bands"], s["ncouls"], s["ngpown"], s["nfreq"], W.FF_SEED)
    schdt = O.ff_schdt(prob).reshape(prob.number_bands, prob.nfreq)
    np.savez_compressed(HERE / "config_ff_schdt.npz", schdt=schdt,
                        meta=np.array([prob.number_bands, prob.ncouls, prob.ngpown, prob.nfreq, W.FF_SEED]))
    print("config_ff_schdt.npz", np.abs(schdt).max(), flush=True)


PARTS = {"production": production, "stress": lambda: production(stress=True), "ff": ff, "batched": batched}

if __name__ == "__main__":
    for part in sys.argv[1:] or list(PARTS):
        t0 = time.time()
        PARTS[part]()
        print(f"{part}: {time.time() - t0:.0f} s", flush=True)
