#!/usr/bin/env python
"""Benchmark of the sigma GPP hot path on GB300.

Workload: the GPP sigma sum of BGW-Kernels/gppKer.cpp at its production shape
(512 bands, nvband 2, ncouls 32768, nodes_per_group 20 -> ngpown 1638, three
frequencies), seeded synthetic inputs (aqsm, aqsn, I_eps ~ U(-1,1) per part,
wtilde re ~ U(0.5,5) im ~ U(-0.1,0.1), vcoul ~ U(0.1,10)) generated on the
device.  One step = one full evaluation of achtemp / asxtemp / acht_n1_loc.

  value      FP64 drop-in, device-resident inputs, Gterms/s
             (terms = number_bands * valid columns * ncouls * 3)
  e2e        the same through the host-pointer C ABI (sigma_gpp_fp64) from
             pinned host buffers: the H2D copy of every input and the D2H of
             the outputs happen inside each timed step
  mixed      the mixed-precision path on the same inputs, its Gterms/s and
             the relative error of every achtemp / asxtemp output against the
             FP64 path (and on the stress fill with 5% near-pole wtilde)
  roofline   the main FP64 kernel (sch_fp64y_kernel): the FP64 pipe work its
             algorithm issues per term (1.34 operations: the FP64 sums of the
             float-float terms plus the shared frequency factor) over
             its CUDA-event time, against the FP64 pipe peak (2 DFMA / clk / SM
             at the SM clock sampled during the timed region); the reference's
             27 flop per term is reported beside it as a rate
  rel_err_vs_oracle  every achtemp / asxtemp output (and acht_n1_loc) of each
             form against the CPU oracle's full outputs of the same seeded
             inputs (tests/golden/config_*.npz)
  cpu_baseline  the reference algorithm (oracle port with the reference's
             loop nest and OpenMP schedule) on a bounded band sample, all host
             cores

--impl reference times the reference's CPU implementation of the same
workload on the host cores (bounded band samples per step) and prints the
same line with "impl": "reference".

Multi-GPU (torchrun): every rank evaluates its own instance (seed 1 + rank)
with no collective on the data path; value is all ranks' terms over the
slowest rank's time (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
for _p in (str(ROOT / "fortkernels-_gb300"), str(ROOT)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "GPP Gterms/s FP64 vs mixed @≤1e-6 rel err, % of measured peak; FF TF/s"
UNIT = "Gterms/s"
WORKLOAD = "GPP sigma sum, FP64 drop-in, 512 bands x 1638 columns x 32768 g-vectors x 3 frequencies"
FLOP_PER_TERM = 27  # algorithmic count of one (n1, igp, ig, iw) term of the reference
CPU_MAX_BANDS = 256
NB, NVB, NC, NPG = 512, 2, 32768, 20
NG = NC // NPG
PRODUCTION = (NB, NVB, NC, NPG)
PER_BAND_WX = False
GOLDEN = ROOT / "tests" / "golden"


def set_shape(nb, nvb, nc, npg):
    """GPP instance shape of the run (the production 512 2 32768 20 by default;
    smaller shapes only for profiling captures)."""
    global NB, NVB, NC, NPG, NG, WORKLOAD
    NB, NVB, NC, NPG = nb, nvb, nc, npg
    NG = NC // NPG
    WORKLOAD = (f"GPP sigma sum, FP64 drop-in, {NB} bands x {NG} columns x {NC} g-vectors x 3 frequencies")


def golden(name):
    """Full oracle outputs of a production workload (None when the fixture is absent)."""
    f = GOLDEN / name
    if not f.exists():
        return None
    with np.load(f) as z:
        return {k: z[k] for k in z.files}


def err_vs_oracle(out, ref):
    """Relative error of every achtemp / asxtemp output, and acht_n1_loc
    normwise, against the oracle's outputs."""
    ach, asx, n1 = out
    e = {"achtemp": rel(ach, ref["achtemp"]), "asxtemp": rel(asx, ref["asxtemp"]),
         "acht_n1_loc_normwise": float(np.linalg.norm(n1 - ref["acht_n1_loc"]) /
                                       np.linalg.norm(ref["acht_n1_loc"]))}
    e["max"] = max(max(e["achtemp"]), max(e["asxtemp"]))
    return e


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={','.join(self.FIELDS)}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------------ CPU baseline
def cpu_sample_problem(seed, bands):
    """Host arrays for the reference CPU code: the last `bands` bands of the
    production instance (non-occupied bands, 99.6% of the terms) and all
    columns, generated with the host twin of the device fill."""
    import workload as W
    lo = NB - bands
    aqsm = np.zeros((NB, NC), np.complex128)
    aqsn = np.zeros((NB, NC), np.complex128)
    aqsm[lo:] = W.fill_complex(seed, W.AID_AQSM, bands * NC, (-1, 1), (-1, 1), start=lo * NC).reshape(bands, NC)
    aqsn[lo:] = W.fill_complex(seed, W.AID_AQSN, bands * NC, (-1, 1), (-1, 1), start=lo * NC).reshape(bands, NC)
    ieps = W.fill_complex(seed, W.AID_IEPS, NG * NC, (-1, 1), (-1, 1)).reshape(NG, NC)
    wt = W.fill_complex(seed, W.AID_WTILDE, NG * NC, (0.5, 5.0), (-0.1, 0.1)).reshape(NG, NC)
    vcoul = W.fill_real(seed, W.AID_VCOUL, NC, 0.1, 10.0)
    inv, indinv = W.gpp_index_maps(NC, NG)
    return W.GppProblem(NB, NVB, NC, NG, inv, indinv, W.wx_frequencies(), aqsm, aqsn, ieps, wt, vcoul)


def time_cpu_reference(prob, band_lo, band_hi, threads):
    from oracle import oracle as O
    t0 = time.perf_counter()
    O.gpp(prob, band_lo, band_hi, nthreads=threads, port=True)
    dt = time.perf_counter() - t0
    terms = (band_hi - band_lo) * NG * NC * 3
    return terms / dt / 1e9, dt


def cpu_baseline(prob, target_s=15.0):
    """Bounded sample of the production workload on all host cores."""
    threads = os.cpu_count() or 1
    calib = 2
    _, dt = time_cpu_reference(prob, NB - calib, NB, threads)
    bands = max(2, min(CPU_MAX_BANDS, int(target_s / (dt / calib))))
    rate, dt = time_cpu_reference(prob, NB - bands, NB, threads)
    return {"value": round(rate, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"bands {NB - bands}..{NB - 1} of the production instance (all 1638 columns, "
                      f"32768 g-vectors, 3 frequencies; {bands * NG * NC * 3:.3e} terms, {dt:.1f} s); "
                      "oracle port of BGW-Kernels/gppKer.cpp:303-439 with its OpenMP dynamic schedule, "
                      "g++ -O3 -fopenmp as the reference builds; the unmodified reference driver only "
                      "runs its constant fill"}


# ------------------------------------------------------------------ reference arm
def run_reference(args, rank):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    prob = cpu_sample_problem(1, 32)
    # size one step to ~3 s of CPU work
    _, dt2 = time_cpu_reference(prob, NB - 2, NB, threads)
    bands = max(1, min(32, int(3.0 / (dt2 / 2))))
    for _ in range(args.warmup):
        time_cpu_reference(prob, NB - bands, NB, threads)
    times = []
    for _ in range(args.steps):
        _, dt = time_cpu_reference(prob, NB - bands, NB, threads)
        times.append(dt)
    terms = bands * NG * NC * 3
    total = sum(times)
    value = terms * len(times) / total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * total / len(times), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "number_bands": NB, "nvband": NVB, "ncouls": NC,
                   "ngpown": NG, "sample_bands_per_step": bands},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{bands} non-occupied bands per step, all columns and g-vectors; "
                                   "the unmodified reference driver only runs its constant fill, so the "
                                   "oracle port of its loop nest (BGW-Kernels/gppKer.cpp:303-439, OpenMP "
                                   "dynamic schedule) runs on the same seeded inputs"},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ our arm
class Instance:
    def __init__(self, S, W, torch, seed, stress=False):
        d = "cuda"
        self.aqsm = torch.empty(2 * NB * NC, dtype=torch.float64, device=d)
        self.aqsn = torch.empty_like(self.aqsm)
        self.ieps = torch.empty(2 * NG * NC, dtype=torch.float64, device=d)
        self.wt = torch.empty_like(self.ieps)
        self.vcoul = torch.empty(NC, dtype=torch.float64, device=d)
        S.fill_complex_device(self.aqsm.data_ptr(), NB * NC, seed, W.AID_AQSM, (-1, 1), (-1, 1))
        S.fill_complex_device(self.aqsn.data_ptr(), NB * NC, seed, W.AID_AQSN, (-1, 1), (-1, 1))
        S.fill_complex_device(self.ieps.data_ptr(), NG * NC, seed, W.AID_IEPS, (-1, 1), (-1, 1))
        S.fill_complex_device(self.wt.data_ptr(), NG * NC, seed, W.AID_WTILDE, (0.5, 5.0), (-0.1, 0.1))
        if stress:
            S.fill_stress_device(self.wt.data_ptr(), NG * NC, seed, W.AID_STRESS, W.wx_frequencies())
        S.fill_real_device(self.vcoul.data_ptr(), NC, seed, W.AID_VCOUL, 0.1, 10.0)
        # PER_BAND_WX: the three frequencies stored once per band (stride 3),
        # which selects the per-band-frequency kernels (profiling captures)
        wx = W.wx_frequencies()
        self.wx_stride = 3 if PER_BAND_WX else 0
        self.wx = torch.tensor(np.tile(wx, NB) if PER_BAND_WX else wx, dtype=torch.float64, device=d)
        self.inv, self.indinv = W.gpp_index_maps(NC, NG)
        self.ach = torch.zeros(6, dtype=torch.float64, device=d)
        self.asx = torch.zeros(6, dtype=torch.float64, device=d)
        self.n1 = torch.zeros(2 * NB, dtype=torch.float64, device=d)

    def run(self, plan, stream):
        plan.execute(self.wx, self.aqsm, self.aqsn, self.ieps, self.wt, self.vcoul, self.ach,
                     self.asx, self.n1, wx_band_stride=self.wx_stride, stream=stream)

    def outputs(self):
        return tuple(t.cpu().numpy().view(np.complex128).copy() for t in (self.ach, self.asx, self.n1))


def rel(a, b):
    return [float(x) for x in (np.abs(a - b) / np.abs(b))]


def timed(torch, dist, world, fn, steps, stream):
    """Runs fn() `steps` times between barriers + synchronize; CUDA-event ms, max over ranks."""
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    if world > 1:
        import replicas
        ms = replicas.max_over_ranks(ms, dist)
    return ms


# FMA-pipe (FP32) lane operations of sch_fp64y_kernel per term, counted from
# its algorithm: 24 paired (f32x2) instructions per term (two products, six
# FMAs of their exact errors and cross terms, one addition, a TwoSum of the
# products, the low sum, a TwoSum into the chunk's float-float sum and two
# additions of its low pair) = 48 lane operations, + the negated high pairs of
# the frequency factors (2 paired per column, frequency and g-vector over 4
# bands: 1 per term) + the chunk-end renormalisation (3 paired per output and
# 16-g-vector chunk: 0.375 per term).
FP64_FMA_LANE_OPS_PER_TERM = 48.0 + 1.0 + 6.0 / 16
# FP64 pipe operations per term: the frequency factor in FP64 (~40 per column
# and g-vector over 64 bands x 3 frequencies = 192 terms) + the chunk-end
# addition of the float-float sums' high pairs (2 per output and 16-g-vector
# chunk).
FP64_PIPE_OPS_PER_TERM = 40.0 / 192 + 2.0 / 16
# ncu, sch_fp64y_kernel, 128-band capture of the production instance
# (--set full): dram__bytes_read.sum + dram__bytes_write.sum per term, and
# sm__pipe_fma_cycles_active / sm__pipe_fp64_cycles_active over elapsed
# cycles.  Traffic scales with the band blocks, so the per-term figure
# carries to the 512-band launch.
FP64_DRAM_BYTES_PER_TERM = 0.1975
FP64_FMA_PIPE_ACTIVE_NCU = 0.713
FP64_PIPE_ACTIVE_NCU = 0.297
# FP32 pipe operations of sch_mixedy_kernel per term: 4 FFMA (complex
# multiply-add) + the float-float fold of each accumulator every 8 g-vectors
# (2 x 7 operations / 8) + the shared frequency factor (~10 per column,
# g-vector and frequency over 64 bands).
MIXED_FP32_OPS_PER_TERM = 4.0 + 14.0 / 8 + 10.0 / 64


FF_SHAPE = (512, 16384, 820, 15)  # number_bands, ncouls, ngpown, nfreq


def library_tensor_rates(torch, n=8192, reps=10):
    """Dense tensor-core rates of this GPU through the vendor library, for
    the choice of slice type of the split contraction: BF16 (torch.matmul)
    and INT8 with INT32 accumulation (torch._int_mm), n^3 GEMMs, best of
    `reps` (CUDA events).  An INT8 split needs about twice the products of
    the BF16 split for the same accuracy (7-bit signed slices against 8-bit
    significands), so it pays only where INT8 runs at more than twice the
    BF16 rate."""
    out = {"n": n}
    for name, make, fn in (
            ("bf16_tflops", lambda: torch.randn(n, n, device="cuda", dtype=torch.bfloat16), torch.matmul),
            ("int8_tops", lambda: torch.randint(-64, 64, (n, n), device="cuda", dtype=torch.int8),
             getattr(torch, "_int_mm", None))):
        if fn is None:
            out[name] = None
            continue
        try:
            a, b = make(), make()
            fn(a, b)
            best = float("inf")
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                fn(a, b)
                e1.record()
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1))
            out[name] = round(2.0 * n ** 3 / (best * 1e-3) / 1e12, 1)
            del a, b
        except RuntimeError as exc:  # no INT8 GEMM for this device in the library
            out[name] = None
            out[name + "_error"] = str(exc).splitlines()[0][:200]
    torch.cuda.empty_cache()
    if out.get("bf16_tflops") and out.get("int8_tops"):
        out["int8_over_bf16"] = round(out["int8_tops"] / out["bf16_tflops"], 3)
    return out


def bf16_peak():
    """Dense BF16 peak for the tensor-core roofline: the measured cuBLAS burst
    figure of this GPU pool (MEASURED_PEAKS.json beside this file), else the
    stated fallback."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 burst; of measured)"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback 1.9 PFLOP/s bf16 burst (no measured peak file; of fallback)"


def run_ff(S, W, torch, dist, world, stream, sptr, args):
    """FF schDt contraction at its production shape: FP64 form and the
    split-BF16 tensor-core form, TF/s = 8 * (nfreq*ngpown) * number_bands *
    ncouls / time, and the tensor form's error against the FP64 form."""
    nb, nc, ng, nf = FF_SHAPE
    epsr = torch.empty(2 * nf * ng * nc, dtype=torch.float64, device="cuda")
    aqsn = torch.empty(2 * nb * nc, dtype=torch.float64, device="cuda")
    aqsm = torch.empty_like(aqsn)
    S.fill_complex_device(epsr.data_ptr(), nf * ng * nc, W.FF_SEED, W.AID_IEPSR, (-1, 1), (-1, 1), sptr)
    S.fill_complex_device(aqsn.data_ptr(), nb * nc, W.FF_SEED, W.AID_AQSN, (-1, 1), (-1, 1), sptr)
    S.fill_complex_device(aqsm.data_ptr(), nb * nc, W.FF_SEED, W.AID_AQSM, (-1, 1), (-1, 1), sptr)
    inv, indinv = W.ff_index_maps(nc, ng)
    flops = 8.0 * nf * ng * nb * nc
    res = {"workload": f"FF schDt: {nb} bands x {nf}x{ng} (ifreq, my_igp) rows x {nc} g-vectors",
           "unit": "TFLOP/s (FP64-equivalent, 8 flop per complex multiply-add)"}
    outs = {}
    for mode, name, steps in ((1, "ozaki_bf16", 20), (0, "fp64", 3)):
        plan = S.FfPlan(nb, nc, ng, nf, inv, indinv, mode)
        out = torch.zeros(2 * nb * nf, dtype=torch.float64, device="cuda")
        for _ in range(2):
            plan.execute(epsr, aqsn, aqsm, out, sptr)
        plan.set_timing(True)
        ms = timed(torch, dist, world, lambda: plan.execute(epsr, aqsn, aqsm, out, sptr), steps, stream)
        t = plan.timing()
        main_s = t["main_ms"] / max(1, t["executions"]) * 1e-3
        res[name] = {"value": round(flops * world / (ms / steps * 1e-3) / 1e12, 3),
                     "ms_per_step": round(ms / steps, 3),
                     "kernel_ms_per_launch": round(main_s * 1e3, 3), "steps": steps,
                     "status": plan.status(sptr)}
        outs[name] = out.cpu().numpy().view(np.complex128)
        plan.close()
    ref = golden("config_ff_schdt.npz") if FF_SHAPE == (512, 16384, 820, 15) else None
    if ref is not None:
        o = ref["schdt"].reshape(-1)
        for name in outs:
            d = outs[name] - o
            res[name]["rel_err_vs_oracle"] = {
                "normwise": float(np.linalg.norm(d) / np.linalg.norm(o)),
                "max_elementwise": float((np.abs(d) / np.abs(o)).max())}
    d = outs["ozaki_bf16"] - outs["fp64"]
    res["ozaki_bf16"]["rel_err_vs_fp64"] = {
        "normwise": float(np.linalg.norm(d) / np.linalg.norm(outs["fp64"])),
        "max_abs_over_max": float(np.abs(d).max() / np.abs(outs["fp64"]).max())}
    res["ozaki_bf16"]["tensor_tflops"] = round(6 * flops / (res["ozaki_bf16"]["kernel_ms_per_launch"] * 1e-3) / 1e12, 1)
    peak, src = bf16_peak()
    res["ozaki_bf16"]["roofline"] = {
        "bound": "tensor", "kernel": "ozaki_gemm_kernel", "achieved": res["ozaki_bf16"]["tensor_tflops"],
        "peak": peak, "unit": "TFLOP/s", "frac": round(res["ozaki_bf16"]["tensor_tflops"] / peak, 4),
        "peak_source": src,
        "note": "achieved = BF16 tensor work (6 slice products of the complex-as-real GEMM, 48 M N K flop) "
                "over the GEMM launch's CUDA-event time"}
    res["speedup_ozaki_vs_fp64"] = round(res["ozaki_bf16"]["value"] / res["fp64"]["value"], 1)
    del epsr, aqsn, aqsm
    torch.cuda.empty_cache()
    return res


FF_SIGMA_NVBAND, FF_SIGMA_NFREQEVAL = 2, 15


def run_ff_sigma(S, W, torch, dist, world, stream, sptr):
    """Full-frequency sigma band loop at the FF production shape (512 bands,
    ncouls 16384, ngpown 820, nfreq 15, nfreqeval 15, nvband 2; seeded
    I_epsR / I_epsA, the mini-app's energies and grid): the two vcoul-weighted
    contractions plus the schDt contraction and the band algebra, in both
    contraction forms; the tensor form's outputs against the FP64 form's."""
    nb, nc, ng, nf = FF_SHAPE
    ne, nv = FF_SIGMA_NFREQEVAL, FF_SIGMA_NVBAND
    f64 = dict(dtype=torch.float64, device="cuda")
    epsr = torch.empty(2 * nf * ng * nc, **f64)
    epsa = torch.empty_like(epsr)
    aqsn = torch.empty(2 * nb * nc, **f64)
    aqsm = torch.empty_like(aqsn)
    vc = torch.empty(nc, **f64)
    S.fill_complex_device(epsr.data_ptr(), nf * ng * nc, W.FF_SEED, W.AID_IEPSR, (-1, 1), (-1, 1), sptr)
    S.fill_complex_device(epsa.data_ptr(), nf * ng * nc, W.FF_SEED, W.AID_IEPSA, (-1, 1), (-1, 1), sptr)
    S.fill_complex_device(aqsn.data_ptr(), nb * nc, W.FF_SEED, W.AID_AQSN, (-1, 1), (-1, 1), sptr)
    S.fill_complex_device(aqsm.data_ptr(), nb * nc, W.FF_SEED, W.AID_AQSM, (-1, 1), (-1, 1), sptr)
    S.fill_real_device(vc.data_ptr(), nc, W.FF_SEED, W.AID_VCOUL, 0.1, 10.0, sptr)
    ekq, grid, brd, pref = W.ff_sigma_grid(nb, nf)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.float64).copy()).cuda()
    d_ekq, d_grid, d_brd, d_pref = dev(ekq), dev(grid), dev(brd.astype(np.complex128)), dev(pref)
    inv, indinv = W.ff_index_maps(nc, ng)
    flops = 3 * 8.0 * nf * ng * nb * nc  # three contractions per step
    res = {"workload": f"FF sigma band loop: {nb} bands x {nf}x{ng} rows x {nc} g-vectors, "
                       f"nfreqeval {ne}, nvband {nv}; 3 contraction outputs (schDt, C_R, C_A) + band "
                       f"algebra per step (the tensor form takes schDt and C_R from one pass)",
           "unit": "TFLOP/s (FP64-equivalent, contractions)"}
    outs = {}
    for mode, name, steps in ((1, "ozaki_bf16", 10), (0, "fp64", 1)):
        plan = S.FfSigmaPlan(nb, nv, nc, ng, nf, ne, inv, indinv, mode)
        out = torch.zeros(2 * (1 + 5 * ne), **f64)
        run = lambda: plan.execute(aqsm, aqsn, epsr, epsa, vc, d_ekq, d_grid, d_brd, d_pref, 0.5 / 3.14, 0.0,
                                   0.5, 1.0, None, out, sptr)
        run()
        plan.set_timing(True)
        ms = timed(torch, dist, world, run, steps, stream)
        t = plan.timing()
        res[name] = {"value": round(flops * world / (ms / steps * 1e-3) / 1e12, 3),
                     "ms_per_step": round(ms / steps, 3),
                     "contraction_ms_per_step": round(t["contraction_ms"] / steps, 3),
                     "status": plan.status(sptr)}
        outs[name] = S.FfSigmaPlan.unpack(out.cpu().numpy(), ne)
        plan.close()
    errs = {}
    for k, v in outs["fp64"].items():
        w = outs["ozaki_bf16"][k]
        errs[k] = float(np.linalg.norm(np.atleast_1d(w - v)) / max(np.linalg.norm(np.atleast_1d(v)), 1e-300))
    res["ozaki_bf16"]["rel_err_vs_fp64_normwise"] = errs
    res["speedup_ozaki_vs_fp64"] = round(res["ozaki_bf16"]["value"] / res["fp64"]["value"], 1)
    del epsr, epsa, aqsn, aqsm
    torch.cuda.empty_cache()
    return res


def run_real(S, W, torch, dist, world, stream, sptr, args):
    """Real-valued GPP (gppKer_real.cpp) at the production shape with seeded
    real inputs (aqsm, aqsn, I_eps ~ U(-1,1), wtilde ~ U(0.5,5), vcoul ~
    U(0.1,10)): FP64 Gterms/s of the device-resident plan."""
    f64 = dict(dtype=torch.float64, device="cuda")
    aqsm = torch.empty(NB * NC, **f64)
    aqsn = torch.empty_like(aqsm)
    ieps = torch.empty(NG * NC, **f64)
    wt = torch.empty_like(ieps)
    vc = torch.empty(NC, **f64)
    seed = W.GPP_PRODUCTION_SEED
    S.fill_real_device(aqsm.data_ptr(), NB * NC, seed, W.AID_AQSM, -1, 1, sptr)
    S.fill_real_device(aqsn.data_ptr(), NB * NC, seed, W.AID_AQSN, -1, 1, sptr)
    S.fill_real_device(ieps.data_ptr(), NG * NC, seed, W.AID_IEPS, -1, 1, sptr)
    S.fill_real_device(wt.data_ptr(), NG * NC, seed, W.AID_WTILDE, 0.5, 5.0, sptr)
    S.fill_real_device(vc.data_ptr(), NC, seed, W.AID_VCOUL, 0.1, 10.0, sptr)
    inv, indinv = W.gpp_index_maps(NC, NG)
    wx = torch.tensor(W.wx_frequencies(), **f64)
    ach, asx, n1 = torch.zeros(3, **f64), torch.zeros(3, **f64), torch.zeros(NB, **f64)
    plan = S.GppRealPlan(NB, NVB, NC, NG, inv, indinv)
    run = lambda: plan.execute(wx, aqsm, aqsn, ieps, wt, vc, ach, asx, n1, stream=sptr)
    for _ in range(args.warmup):
        run()
    steps = max(args.steps, 5)
    ms = timed(torch, dist, world, run, steps, stream)
    plan.close()
    terms = NB * NG * NC * 3
    res = {"workload": f"real-valued GPP, {NB} bands x {NG} columns x {NC} g-vectors x 3 frequencies, FP64",
           "value": round(terms * world / (ms / steps * 1e-3) / 1e9, 4), "unit": UNIT,
           "ms_per_step": round(ms / steps, 3), "steps": steps}
    del aqsm, aqsn, ieps, wt
    torch.cuda.empty_cache()
    return res


def run_halfsum(S, W, torch, dist, world, stream, sptr, args, inst):
    """gppsum = 1 half sum (gppKerSeq.cpp) on the production instance's device
    arrays, FP64: Gterms/s of the band sums (terms = bands x sum over valid
    columns of igp x 3, the (n1, my_igp, ig < igp, iw) iterations of the
    reference's loop), and the step time with the static remainder."""
    f64 = dict(dtype=torch.float64, device="cuda")
    igp = np.array([NC - 1 if i == NC else int(inst.indinv[i]) for i in inst.inv])
    igp = igp[igp >= 0]
    terms = NB * int(igp.sum()) * 3
    ach, asx, n1, st = (torch.zeros(6, **f64), torch.zeros(6, **f64), torch.zeros(2 * NB, **f64),
                        torch.zeros(2, **f64))
    res = {"workload": f"gppsum=1 half sum, {NB} bands x {NG} columns x g-vectors below igp "
                       f"(of {NC}) x 3 frequencies, FP64, band-major device arrays",
           "unit": UNIT, "terms_per_step": terms}
    outs = {}
    forms = args.halfsum_forms.split(",")
    for flags, key, steps in ((0, "sums", 3), (S.HALFSUM_STATIC, "with_static", 3),
                              (S.HALFSUM_STATIC | S.HALFSUM_TENSOR, "tensor", 10)):
        if key not in forms:
            continue
        plan = S.GppHalfSumPlan(NB, NVB, NC, NG, inst.inv, inst.indinv, flags=flags)
        run = lambda: plan.execute(inst.wx, inst.aqsm, inst.aqsn, inst.ieps, inst.wt, inst.vcoul, ach, asx,
                                   n1, st if flags else None, stream=sptr)
        for _ in range(max(1, min(args.warmup, 2))):
            run()
        ms = timed(torch, dist, world, run, steps, stream)
        plan.close()
        outs[key] = [t.cpu().numpy().view(np.complex128).copy() for t in (ach, asx, n1, st)]
        if key == "sums":
            res["value"] = round(terms * world / (ms / steps * 1e-3) / 1e9, 4)
            res["ms_per_step"] = round(ms / steps, 3)
        elif key == "with_static":
            res["with_static_ms_per_step"] = round(ms / steps, 3)
        else:
            a, b = outs["tensor"], outs.get("with_static")
            res["tensor"] = {
                "value": round(terms * world / (ms / steps * 1e-3) / 1e9, 4), "unit": UNIT,
                "ms_per_step_with_static": round(ms / steps, 3),
                "rel_err_vs_fp64": None if b is None else {"achtemp": rel(a[0], b[0]), "asxtemp": rel(a[1], b[1]),
                                    "achstemp": float(abs(a[3][0] - b[3][0]) / abs(b[3][0])),
                                    "acht_n1_loc_normwise": float(np.linalg.norm(a[2] - b[2]) /
                                                                  np.linalg.norm(b[2]))},
                "path": "band sums as four split-BF16 tcgen05 contractions (T, U, static T and U) of "
                        "FP32 factor slabs formed in float-float arithmetic; occupied bands with "
                        "float-float factors, FP32 products and float-float sums; unpaired igp terms "
                        "in FP64"}
    return res


def run_static(S, W, torch, dist, world, stream, sptr, inst):
    """Static remainder (sigma_gpp_static_execute) on the production
    instance's device arrays: both contraction forms, FP64-equivalent TF/s
    (8 flop per complex multiply-add of the bands x columns x g-vectors
    GEMM) and the tensor form's error against the FP64 form."""
    flops = 8.0 * NB * NG * NC
    res = {"workload": f"GPP static remainder: {NB} bands x {NG} columns x {NC} g-vectors",
           "unit": "TFLOP/s (FP64-equivalent)"}
    outs = {}
    for mode, name, steps in ((1, "ozaki_bf16", 10), (0, "fp64", 2)):
        plan = S.StaticPlan(NB, NC, NG, inst.inv, inst.indinv, mode)
        tot = torch.zeros(2, dtype=torch.float64, device="cuda")
        n1 = torch.zeros(2 * NB, dtype=torch.float64, device="cuda")
        run = lambda: plan.execute(inst.aqsm, inst.aqsn, inst.ieps, inst.vcoul, tot, n1, sptr)
        run()
        plan.set_timing(True)
        ms = timed(torch, dist, world, run, steps, stream)
        t = plan.timing()
        res[name] = {"value": round(flops * world / (ms / steps * 1e-3) / 1e12, 3),
                     "ms_per_step": round(ms / steps, 3),
                     "kernel_ms_per_launch": round(t["main_ms"] / max(1, t["executions"]), 3),
                     "status": plan.status(sptr)}
        outs[name] = (tot.cpu().numpy().view(np.complex128)[0], n1.cpu().numpy().view(np.complex128).copy())
        plan.close()
    a, b = outs["fp64"], outs["ozaki_bf16"]
    res["ozaki_bf16"]["rel_err_vs_fp64"] = {"achstemp": float(abs(b[0] - a[0]) / abs(a[0])),
                                            "per_band_normwise": float(np.linalg.norm(b[1] - a[1]) /
                                                                       np.linalg.norm(a[1]))}
    res["speedup_ozaki_vs_fp64"] = round(res["ozaki_bf16"]["value"] / res["fp64"]["value"], 1)
    return res


def time_single_plans(S, torch, dist, world, xs, prec, stream):
    """The same instances as one device-resident plan each, executed back to
    back on one stream (plans created and warmed up outside the timed
    region): ms for one pass over all of them."""
    f64 = dict(dtype=torch.float64, device="cuda")
    plans = [S.GppPlan(x.nb, x.nvb, x.nc, x.ng, x.inv, x.indinv, precision=prec) for x in xs]
    outs = [(torch.zeros(6, **f64), torch.zeros(6, **f64), torch.zeros(2 * x.nb, **f64)) for x in xs]
    sp = stream.cuda_stream

    def one_pass():
        for x, pl, o in zip(xs, plans, outs):
            pl.execute(x.wx, x.aqsm, x.aqsn, x.ieps, x.wt, x.vcoul, *o, stream=sp)

    one_pass()
    ms = timed(torch, dist, world, one_pass, 1, stream)
    for pl in plans:
        pl.close()
    torch.cuda.empty_cache()
    return ms


def run_batched(S, W, torch, dist, world, stream, sptr, args, dropin_value):
    """48 uneven GPP instances (workload.batched_shapes) through the batched
    API, one CUDA-graph replay per step, FP64 (tiles from the tuning table)
    and mixed; Gterms/s over the whole batch and the mixed outputs' error
    against the FP64 ones."""
    import autotune
    import batched

    shapes = W.batched_shapes()[: args.batch_instances]
    xs = batched.device_instances(shapes)
    dicts = [x.as_dict() for x in xs]
    tiles = [autotune.tile_for(x.nb, x.ng, shared=True) for x in xs]
    res = {"workload": f"{len(xs)} GPP instances, number_bands U{{64..512}}, ncouls U{{4096..32768}}/256, "
                       "nodes_per_group U{10..40}, nvband U{1..8}, seeds 1000+i",
           "instances": len(xs), "input_bytes": int(sum(x.input_bytes for x in xs)),
           "tiles": {"table": autotune.load_table() is not None,
                     "counts": {autotune.TILES[t] if t >= 0 else "library": tiles.count(t)
                                for t in sorted(set(tiles))},
                     "items_per_cta": {f: autotune.sizing_for(f) for f in ("fp64", "mixed")},
                     "tensor_split_tiles": autotune.sizing_for("tensor")}}
    outs = {}
    gs = torch.cuda.Stream()  # graphs are captured on a non-default stream
    gptr = gs.cuda_stream
    torch.cuda.synchronize()
    forms = [(S.PREC_FP64, "fp64", args.batch_fp64_steps), (S.PREC_MIXED, "mixed", 5),
             (S.PREC_TENSOR, "tensor", 5)]
    forms = [f for f in forms if f[1] in args.batch_forms.split(",")]
    for prec, name, steps in forms:
        b = S.GppBatch(dicts, precision=prec, tiles=tiles if prec == S.PREC_FP64 else None,
                       items_per_cta=autotune.sizing_for(name) if name != "tensor" else 0,
                       tensor_split_tiles=autotune.sizing_for("tensor") if name == "tensor" else 0)
        terms, items, launches = b.info()
        b.launch_graph(gptr)  # capture, and the warm-up replay
        ms = timed(torch, dist, world, lambda: b.launch_graph(gptr), steps, gs)
        st = b.status(gptr)
        outs[name] = [x.outputs() for x in xs]
        res[name] = {"value": round(terms * world / (ms / steps * 1e-3) / 1e9, 4), "unit": UNIT,
                     "ms_per_step": round(ms / steps, 3), "steps": steps, "terms_per_step": terms,
                     "items": items, "kernels_per_step": launches, "status": st}
        b.close()
        torch.cuda.empty_cache()
        if not args.no_batch_singles:
            single_ms = time_single_plans(S, torch, dist, world, xs, prec, gs)
            res[name]["single_plans_ms_per_step"] = round(single_ms, 3)
            res[name]["batch_over_single_plans_time"] = round((ms / steps) / single_ms, 4)
    ref = golden("config_gpp_batched.npz")
    if ref is not None:
        off = ref["n1_offsets"]
        for name in outs:
            worst, over, n1_worst, at = 0.0, 0, 0.0, ""
            n1_band_worst, n1_band_at = 0.0, ""
            by = {"achtemp": 0.0, "asxtemp": 0.0}
            for i, o in enumerate(outs[name]):
                for k, key in ((0, "achtemp"), (1, "asxtemp")):
                    e = np.abs(o[k] - ref[key][i]) / np.abs(ref[key][i])
                    if float(e.max()) > worst:
                        worst, at = float(e.max()), f"instance {i} {key}[{int(np.argmax(e))}]"
                    by[key] = max(by[key], float(e.max()))
                    over += int(np.sum(e > (1e-12 if name == "fp64" else 1e-6)))
                r1 = ref["acht_n1_loc"][off[i]:off[i + 1]]
                n1_worst = max(n1_worst, float(np.linalg.norm(o[2] - r1) / np.linalg.norm(r1)))
                # per band, over the bands the tests bound relatively (at
                # least 1e-3 of the instance's largest band value)
                big = np.abs(r1) >= 1e-3 * np.abs(r1).max()
                eb = np.abs(o[2][big] - r1[big]) / np.abs(r1[big])
                if eb.size and float(eb.max()) > n1_band_worst:
                    n1_band_worst = float(eb.max())
                    n1_band_at = f"instance {i} band {int(np.nonzero(big)[0][int(np.argmax(eb))])}"
            res[name]["rel_err_vs_oracle"] = {"max": worst, "max_at": at, "max_by_output": by,
                                              "outputs_over_bar": over,
                                              "bar": 1e-12 if name == "fp64" else 1e-6,
                                              "outputs": 6 * len(outs[name]),
                                              "acht_n1_loc_normwise_max": n1_worst,
                                              "acht_n1_loc_band_max": n1_band_worst,
                                              "acht_n1_loc_band_max_at": n1_band_at}
    for name in ("mixed", "tensor"):
        if name not in outs or "fp64" not in outs:
            continue
        worst, over, by = 0.0, 0, {"achtemp": 0.0, "asxtemp": 0.0}
        for a, m in zip(outs["fp64"], outs[name]):
            for k, key in ((0, "achtemp"), (1, "asxtemp")):
                e = np.abs(m[k] - a[k]) / np.abs(a[k])
                worst = max(worst, float(e.max()))
                by[key] = max(by[key], float(e.max()))
                over += int(np.sum(e > 1e-6))
        res[name]["max_rel_err_vs_fp64"] = worst
        res[name]["max_rel_err_vs_fp64_by_output"] = by
        res[name]["outputs_over_1e-6"] = over
        res[name]["outputs"] = 6 * len(xs)
        res[name]["speedup_vs_fp64_batched"] = round(res[name]["value"] / res["fp64"]["value"], 2)
        res[name]["speedup_vs_fp64_dropin"] = round(res[name]["value"] / dropin_value, 2)
    del xs, dicts
    torch.cuda.empty_cache()
    return res


def run_ours(args, rank, world, local_rank):
    import torch
    import sigma_gb300 as S
    import workload as W

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    S.load()
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    if args.only_batched:
        res = run_batched(S, W, torch, dist, world, stream, sptr, args, float("nan"))
        if rank == 0:
            print(json.dumps({"batched": res}), flush=True)
        return 0
    if args.only_ff:
        res = run_ff(S, W, torch, dist, world, stream, sptr, args)
        if rank == 0:
            print(json.dumps({"ff": res}), flush=True)
        return 0
    if args.only_ff_sigma:
        res = run_ff_sigma(S, W, torch, dist, world, stream, sptr)
        if rank == 0:
            print(json.dumps({"ff_sigma": res}), flush=True)
        return 0
    if args.only_gpp_forms:
        import replicas
        inst = Instance(S, W, torch, seed=replicas.rank_seed(W.GPP_PRODUCTION_SEED, rank))
        res = {}
        for name in args.only_gpp_forms.split(","):
            prec = {"fp64": S.PREC_FP64, "mixed": S.PREC_MIXED, "tensor": S.PREC_TENSOR}[name]
            pl = S.GppPlan(NB, NVB, NC, NG, inst.inv, inst.indinv, precision=prec)
            _, terms = pl.info()
            for _ in range(args.warmup):
                inst.run(pl, sptr)
            ms = timed(torch, dist, world, lambda: inst.run(pl, sptr), args.steps, stream)
            pl.close()
            res[name] = {"value": round(terms * world / (ms / args.steps * 1e-3) / 1e9, 4), "unit": UNIT,
                         "ms_per_step": round(ms / args.steps, 3)}
        if rank == 0:
            print(json.dumps({"gpp_forms": res, "per_band_wx": PER_BAND_WX}), flush=True)
        return 0
    if args.only_gpp_tensor:
        import replicas
        inst = Instance(S, W, torch, seed=replicas.rank_seed(W.GPP_PRODUCTION_SEED, rank))
        tplan = S.GppPlan(NB, NVB, NC, NG, inst.inv, inst.indinv, precision=S.PREC_TENSOR)
        _, terms = tplan.info()
        for _ in range(args.warmup):
            inst.run(tplan, sptr)
        ms = timed(torch, dist, world, lambda: inst.run(tplan, sptr), args.steps, stream)
        tplan.close()
        if rank == 0:
            print(json.dumps({"tensor": {"value": round(terms * world / (ms / args.steps * 1e-3) / 1e9, 4),
                                         "unit": UNIT, "ms_per_step": round(ms / args.steps, 3)}}), flush=True)
        return 0
    if args.only_halfsum:
        import replicas
        inst = Instance(S, W, torch, seed=replicas.rank_seed(W.GPP_PRODUCTION_SEED, rank))
        res = run_halfsum(S, W, torch, dist, world, stream, sptr, args, inst)
        if rank == 0:
            print(json.dumps({"halfsum": res}), flush=True)
        return 0
    fp64_peak, fp32_peak = S.measure_fma_peaks(sptr)
    lib_rates = None if args.no_ff else library_tensor_rates(torch)
    import replicas
    inst = Instance(S, W, torch, seed=replicas.rank_seed(W.GPP_PRODUCTION_SEED, rank))
    plan = S.GppPlan(NB, NVB, NC, NG, inst.inv, inst.indinv, precision=S.PREC_FP64)
    valid, terms = plan.info()

    # ---- device-resident FP64 drop-in
    for _ in range(args.warmup):
        inst.run(plan, sptr)
    plan.set_timing(True)
    clocks = ClockSampler(local_rank)
    clocks.start()
    ms = timed(torch, dist, world, lambda: inst.run(plan, sptr), args.steps, stream)
    clk = clocks.stop()
    kt = plan.timing()
    plan.set_timing(False)
    fp64_out = inst.outputs()
    ms_step = ms / args.steps
    value = terms * world / (ms_step * 1e-3) / 1e9
    main_s = kt["main_ms"] / max(1, kt["executions"]) * 1e-3
    algorithmic_tflops = FLOP_PER_TERM * terms / main_s / 1e12
    pipe_tflops = 2 * FP64_FMA_LANE_OPS_PER_TERM * terms / main_s / 1e12
    fp64_pipe_tflops = 2 * FP64_PIPE_OPS_PER_TERM * terms / main_s / 1e12
    production = (NB, NVB, NC, NPG) == PRODUCTION
    ref_prod = golden("config_gpp_production.npz") if production else None
    ref_stress = golden("config_gpp_stress.npz") if production else None

    # ---- end to end through the host C ABI (pinned host buffers)
    host = {k: torch.empty(getattr(inst, k).numel(), dtype=torch.float64, pin_memory=True)
            for k in ("aqsm", "aqsn", "ieps", "wt", "vcoul")}
    for k, t in host.items():
        t.copy_(getattr(inst, k))
    inv = np.ascontiguousarray(inst.inv, np.int32)
    indinv = np.ascontiguousarray(inst.indinv, np.int32)
    wx = np.ascontiguousarray(W.wx_frequencies())
    h_ach = torch.zeros(6, dtype=torch.float64, pin_memory=True)
    h_asx = torch.zeros(6, dtype=torch.float64, pin_memory=True)
    h_n1 = torch.zeros(2 * NB, dtype=torch.float64, pin_memory=True)
    lib = S.load()

    def e2e_step():
        st = lib.sigma_gpp_fp64(NB, NVB, NC, NG, 0, 3, inv.ctypes.data, indinv.ctypes.data,
                                wx.ctypes.data, 1.0, host["aqsm"].data_ptr(), host["aqsn"].data_ptr(),
                                host["ieps"].data_ptr(), host["wt"].data_ptr(), host["vcoul"].data_ptr(),
                                h_ach.data_ptr(), h_asx.data_ptr(), h_n1.data_ptr(), sptr)
        if st != 0:
            raise S.SigmaError(st, "sigma_gpp_fp64")

    e2e_steps = max(1, min(args.steps, 5))
    if args.no_e2e:
        e2e_steps, ms_e2e = 0, float("nan")
    else:
        for _ in range(min(args.warmup, 2)):
            e2e_step()
        ms_e2e = timed(torch, dist, world, e2e_step, e2e_steps, stream)
    e2e_value = terms * world / (ms_e2e / max(1, e2e_steps) * 1e-3) / 1e9
    h2d = sum(t.numel() * 8 for t in host.values()) + wx.nbytes
    d2h = (6 + 6 + 2 * NB) * 8
    e2e_match = bool(np.array_equal(h_ach.numpy().view(np.complex128), fp64_out[0])) if e2e_steps else None
    del host
    S.shutdown()  # frees the drop-in's cached device copy of the inputs

    # ---- mixed precision on the same inputs, then the stress fill
    mplan = S.GppPlan(NB, NVB, NC, NG, inst.inv, inst.indinv, precision=S.PREC_MIXED)
    for _ in range(args.warmup):
        inst.run(mplan, sptr)
    mplan.set_timing(True)
    msteps = max(args.steps, 10)
    ms_mixed = timed(torch, dist, world, lambda: inst.run(mplan, sptr), msteps, stream)
    mkt = mplan.timing()
    mixed_out = inst.outputs()
    mixed_value = terms * world / (ms_mixed / msteps * 1e-3) / 1e9
    mixed_err = {"achtemp": rel(mixed_out[0], fp64_out[0]), "asxtemp": rel(mixed_out[1], fp64_out[1]),
                 "acht_n1_loc_normwise": float(np.linalg.norm(mixed_out[2] - fp64_out[2]) /
                                               np.linalg.norm(fp64_out[2]))}
    mixed_main_s = mkt["main_ms"] / max(1, mkt["executions"]) * 1e-3
    mixed_pipe = 2 * MIXED_FP32_OPS_PER_TERM * terms / mixed_main_s / 1e12

    # ---- tensor-core form on the same inputs
    tplan = S.GppPlan(NB, NVB, NC, NG, inst.inv, inst.indinv, precision=S.PREC_TENSOR)
    for _ in range(args.warmup):
        inst.run(tplan, sptr)
    tplan.set_timing(True)
    tsteps = max(args.steps, 10)
    ms_tensor = timed(torch, dist, world, lambda: inst.run(tplan, sptr), tsteps, stream)
    tkt = tplan.timing()
    tensor_out = inst.outputs()
    tensor_value = terms * world / (ms_tensor / tsteps * 1e-3) / 1e9
    tensor_err = {"achtemp": rel(tensor_out[0], fp64_out[0]), "asxtemp": rel(tensor_out[1], fp64_out[1]),
                  "acht_n1_loc_normwise": float(np.linalg.norm(tensor_out[2] - fp64_out[2]) /
                                                np.linalg.norm(fp64_out[2]))}
    static = None if args.no_static else run_static(S, W, torch, dist, world, stream, sptr, inst)
    half = None if args.no_halfsum else run_halfsum(S, W, torch, dist, world, stream, sptr, args, inst)
    cpu_prob = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # host copy of the instance for the CPU baseline: trailing bands + all columns
        nkeep = min(NB, CPU_MAX_BANDS)
        c = lambda t, r: t.view(-1, 2).cpu().numpy().view(np.complex128).reshape(r, NC)
        aqsm = np.zeros((NB, NC), np.complex128)
        aqsn = np.zeros((NB, NC), np.complex128)
        aqsm[NB - nkeep:] = c(inst.aqsm, NB)[NB - nkeep:]
        aqsn[NB - nkeep:] = c(inst.aqsn, NB)[NB - nkeep:]
        cpu_prob = W.GppProblem(NB, NVB, NC, NG, inst.inv, inst.indinv, W.wx_frequencies(), aqsm, aqsn,
                                c(inst.ieps, NG), c(inst.wt, NG), inst.vcoul.cpu().numpy())
    del inst
    torch.cuda.empty_cache()
    sinst = Instance(S, W, torch, seed=W.GPP_STRESS_SEED, stress=True)
    sinst.run(plan, sptr)
    s64 = sinst.outputs()
    sinst.run(mplan, sptr)
    smx = sinst.outputs()
    stress_err = {"achtemp": rel(smx[0], s64[0]), "asxtemp": rel(smx[1], s64[1])}
    sinst.run(tplan, sptr)
    stc = sinst.outputs()
    tensor_stress_err = {"achtemp": rel(stc[0], s64[0]), "asxtemp": rel(stc[1], s64[1])}
    oracle = None
    if ref_prod is not None and ref_stress is not None:
        forms = {"fp64": (fp64_out, s64), "mixed": (mixed_out, smx), "tensor": (tensor_out, stc)}
        oracle = {k: {"production": err_vs_oracle(a, ref_prod), "stress": err_vs_oracle(b, ref_stress)}
                  for k, (a, b) in forms.items()}
        for k, v in oracle.items():
            v["max"] = max(v["production"]["max"], v["stress"]["max"])
            v["bar"] = 1e-12 if k == "fp64" else 1e-6
            v["within_bar"] = v["max"] <= v["bar"]
    tplan.close()
    del sinst
    plan.close()
    mplan.close()
    torch.cuda.empty_cache()

    props = torch.cuda.get_device_properties(local_rank)
    sms = props.multi_processor_count
    clock_mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
    # FP64 pipe: 2 DFMA / clk / SM, FP32: 128 FFMA / clk / SM (ncu peak_sustained on GB300)
    fp64_pipe_peak = 2 * 2 * sms * clock_mhz * 1e6 / 1e12
    fp32_pipe_peak = 2 * 128 * sms * clock_mhz * 1e6 / 1e12
    ff = None if args.no_ff else run_ff(S, W, torch, dist, world, stream, sptr, args)
    ffs = None if args.no_ff else run_ff_sigma(S, W, torch, dist, world, stream, sptr)
    real = None if args.no_real else run_real(S, W, torch, dist, world, stream, sptr, args)
    batch = None if args.no_batched else run_batched(S, W, torch, dist, world, stream, sptr, args, value)
    worst = max(max(mixed_err["achtemp"]), max(mixed_err["asxtemp"]),
                max(stress_err["achtemp"]), max(stress_err["asxtemp"]))
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded SplitMix64 fill of the production shape; no dataset exists)",
        "config": {"workload": WORKLOAD, "number_bands": NB, "nvband": NVB, "ncouls": NC,
                   "nodes_per_group": NPG, "ngpown": NG, "valid_columns": valid,
                   "terms_per_step": terms, "l2": "inputs (2.25 GB) larger than L2 (129 MB)",
                   "parallelism": f"replicas x{world} (one independent instance per GPU)"},
        "e2e": {"value": (round(e2e_value, 4) if e2e_steps else None), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                "path": "sigma_gpp_fp64 host C ABI, pinned buffers", "matches_device_path": e2e_match},
        "roofline": {"bound": "fp32_pipe", "kernel": "sch_fp64y_kernel",
                     "achieved": round(pipe_tflops, 4), "peak": round(fp32_pipe_peak, 4), "unit": "TFLOP/s",
                     "frac": round(pipe_tflops / fp32_pipe_peak, 4),
                     "traffic": round(FP64_DRAM_BYTES_PER_TERM * terms),
                     "kernel_ms_per_launch": round(main_s * 1e3, 3),
                     "fma_lane_ops_per_term": round(FP64_FMA_LANE_OPS_PER_TERM, 4),
                     "peak_source": f"FMA pipe 128 lanes/clk/SM x {sms} SMs x {clock_mhz:.0f} MHz, 2 flop "
                                    "per lane operation (SM clock sampled during the timed region; the "
                                    "measured-peaks file has no FP32 figure)",
                     "ncu_fma_pipe_active": FP64_FMA_PIPE_ACTIVE_NCU,
                     "fp64_pipe": {"achieved": round(fp64_pipe_tflops, 4), "peak": round(fp64_pipe_peak, 4),
                                   "frac": round(fp64_pipe_tflops / fp64_pipe_peak, 4),
                                   "ops_per_term": round(FP64_PIPE_OPS_PER_TERM, 4),
                                   "ncu_active": FP64_PIPE_ACTIVE_NCU,
                                   "peak_source": f"FP64 pipe 2 DFMA/clk/SM x {sms} SMs at the sampled clock; "
                                                  f"dependent-FMA probe on this device: {fp64_peak:.3f} TFLOP/s"},
                     "algorithmic": {"flop_per_term": FLOP_PER_TERM,
                                     "tflops": round(algorithmic_tflops, 4),
                                     "note": "the reference's 27 flop per term (its own formulation, which "
                                             "rebuilds the frequency factor for every band) at the measured "
                                             "term rate: a rate, not a pipe fraction"},
                     "note": "achieved = FMA-pipe work of the kernel's own algorithm (each lane operation "
                             "one FMA slot, 2 flop): with one frequency set for all bands the frequency "
                             "factor is formed in FP64 once per column and g-vector and split to float-float; "
                             "every term is a float-float product in paired FP32 instructions (real and "
                             "imaginary parts as the two lanes), added exactly (TwoSum) to a per-chunk "
                             "float-float sum whose high pair is added to the FP64 sums every 16 g-vectors; "
                             "the FP64 pipe carries the factor and those additions (fp64_pipe); "
                             "traffic = ncu DRAM bytes per term x terms"},
        "rel_err_vs_oracle": oracle,
        "mixed": {"value": round(mixed_value, 4), "unit": UNIT,
                  "speedup_vs_fp64": round(mixed_value / value, 3),
                  "ms_per_step": round(ms_mixed / msteps, 3),
                  "kernel_ms_per_launch": round(mixed_main_s * 1e3, 3),
                  "rel_err_vs_fp64": mixed_err, "stress_rel_err_vs_fp64": stress_err,
                  "max_rel_err": worst, "within_1e-6": worst <= 1e-6,
                  "roofline": {"bound": "fp32_pipe", "kernel": "sch_mixedy_kernel",
                               "achieved": round(mixed_pipe, 3),
                               "peak": round(fp32_pipe_peak, 3), "unit": "TFLOP/s",
                               "frac": round(mixed_pipe / fp32_pipe_peak, 4),
                               "fp32_pipe_ops_per_term": round(MIXED_FP32_OPS_PER_TERM, 4),
                               "algorithmic_tflops_27_flop_per_term":
                                   round(FLOP_PER_TERM * terms / mixed_main_s / 1e12, 3),
                               "peak_source": "FP32 pipe 128 FFMA/clk/SM at the sampled SM clock",
                               "note": "achieved = FP32 pipe work (2 flop per FFMA) of the kernel's own "
                                       "algorithm: 4 FFMA per term for the complex multiply-add, the "
                                       "float-float fold every 8 g-vectors and the shared frequency factor"}},
        "tensor": {"value": round(tensor_value, 4), "unit": UNIT,
                   "speedup_vs_fp64": round(tensor_value / value, 3),
                   "ms_per_step": round(ms_tensor / tsteps, 3),
                   "main_ms_per_step": round(tkt["main_ms"] / max(1, tkt["executions"]), 3),
                   "rel_err_vs_fp64": tensor_err, "stress_rel_err_vs_fp64": tensor_stress_err,
                   "max_rel_err": max(max(tensor_err["achtemp"]), max(tensor_err["asxtemp"]),
                                      max(tensor_stress_err["achtemp"]), max(tensor_stress_err["asxtemp"])),
                   "path": "one factor pass: frequency factors in float-float arithmetic on the FP32 pipe, "
                           "rounded to FP32 and written as the contraction's split-BF16 slices, with the "
                           "occupied bands' sums, the B slices and the epilogue factors; band sum as "
                           "split-BF16 tcgen05 GEMM"},
        "ff": ff,
        "ff_sigma": ffs,
        "batched": batch,
        "static_remainder": static,
        "real": real,
        "halfsum": half,
        "peaks_measured": {"fp64_fma_probe_tflops": round(fp64_peak, 4),
                           "fp32_fma_probe_tflops": round(fp32_peak, 3),
                           "fp64_pipe_tflops_at_clock": round(fp64_pipe_peak, 4),
                           "fp32_pipe_tflops_at_clock": round(fp32_pipe_peak, 3),
                           "library_tensor_rates": lib_rates},
        "clocks": clk,
        "gpu_launches": int(kt["launches"]) * args.steps,
    }
    if cpu_prob is not None:
        line["cpu_baseline"] = cpu_baseline(cpu_prob)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-ff", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-static", action="store_true")
    ap.add_argument("--no-real", action="store_true")
    ap.add_argument("--no-halfsum", action="store_true")
    ap.add_argument("--only-gpp-tensor", action="store_true",
                    help="run the tensor-core GPP measurement alone (profiling captures)")
    ap.add_argument("--only-halfsum", action="store_true",
                    help="run the gppsum=1 half-sum measurement alone (profiling captures)")
    ap.add_argument("--halfsum-forms", default="sums,with_static,tensor",
                    help="half-sum forms to time: sums (FP64), with_static (FP64 with the static "
                         "remainder), tensor; the tensor form's error needs with_static")
    ap.add_argument("--ff-shape", default=None,
                    help="number_bands,ncouls,ngpown,nfreq of the FF runs (default the production "
                         "512,16384,820,15; smaller only for profiling captures)")
    ap.add_argument("--only-ff", action="store_true", help="run the FF contraction alone (profiling)")
    ap.add_argument("--only-ff-sigma", action="store_true",
                    help="run the FF band loop alone at --ff-shape (profiling)")
    ap.add_argument("--batch-instances", type=int, default=48,
                    help="leading instances of the 48-instance batched set (fewer only for profiling)")
    ap.add_argument("--batch-fp64-steps", type=int, default=2)
    ap.add_argument("--no-batch-singles", action="store_true",
                    help="skip timing the batched instances as single plans back to back")
    ap.add_argument("--batch-forms", default="fp64,mixed,tensor",
                    help="comma list of the batched forms to time (fewer only for profiling)")
    ap.add_argument("--only-batched", action="store_true",
                    help="run the batched measurement alone (profiling captures)")
    ap.add_argument("--per-band-wx", action="store_true",
                    help="frequencies stored per band (the per-band-frequency kernels; FP64 and mixed "
                         "only, for profiling captures)")
    ap.add_argument("--only-gpp-forms", default=None,
                    help="comma list of fp64,mixed,tensor: run those plans alone on the instance "
                         "(profiling captures)")
    ap.add_argument("--gpp-shape", default=None,
                    help="number_bands,nvband,ncouls,nodes_per_group of the GPP instance (default the "
                         "production 512,2,32768,20; smaller only for profiling captures)")
    args = ap.parse_args()
    if args.gpp_shape:
        set_shape(*(int(x) for x in args.gpp_shape.split(",")))
    global PER_BAND_WX
    PER_BAND_WX = args.per_band_wx
    if args.ff_shape:
        global FF_SHAPE
        FF_SHAPE = tuple(int(x) for x in args.ff_shape.split(","))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)
    return run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
