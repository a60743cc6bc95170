"""Regenerates the golden fixtures from the reference itself.

Needs the reference checkout (REFERENCE_ROOT; oracle/build.py, the build
recipe that reads it, gives the default location); the
fixtures it writes are committed so the tests run without it.

  gpp_reference_constfill.json  achtemp printed by the unmodified
      BGW-Kernels/gppKer.cpp driver (constant fill) at several shapes and
      OpenMP thread counts, plus the closed form of the constant fill.
  gpp_flagocc_<case>.npz        ssx_array / sch_array per (band, column,
      frequency) from the reference's own flagOCC_solver
      (BGW-Kernels/gppKer.cpp:130-159) on seeded inputs that
      fortkernels-_gb300/workload.py regenerates from the recorded seed.

  ff_sigma_reference.json       the unmodified FFKer_cori/ffKernel.cpp
      driver's printed achsDtemp / asxDtemp(1) / achDtemp_cor(1) on its
      constant fill, and its achsDtemp_Kernel / asxDtemp_Kernel /
      achDtemp_cor_Kernel (through oracle/ff_ref_harness.cpp) on seeded
      inputs that workload.ff_sigma_random regenerates.  The C++ kernels
      differ from the Fortran loop in places that these inputs avoid or
      undo (recorded per case): achsDtemp_Kernel reads frequency 1 (the
      Fortran frequency 1 is index 0), so slab 1 holds slab 0; wx lacks the
      (iw-1) * freqevalstep term, so the C++ kernels run with freqevalmin
      one step lower and every iw equals the Fortran iw = 0; no wx falls on
      a grid point or outside the grid, where the C++ interval search
      differs.

  gpp_real_reference.json       the unmodified gppKer_real.cpp driver's
      printed achtemp (15 digits) on its constant fill; gpp_real_flagocc_<case>.npz
      ssx_array / sch_array per (band, column, frequency) from its own
      flagOCC_solver on seeded inputs (workload.gpp_real_random).

  gpp_halfsum_reference.json    the unmodified gppKerSeq.cpp driver (the
      reference's one buildable statement of gppsum = 1) run with gppsum = 1:
      its printed achtemp (15 digits) on its constant fill.
      gpp_halfsum_<case>.npz sch_array / ssx_array per (band, column,
      frequency) from its own flagOCC_solver / noflagOCC_solver, driven in
      the 512-wide g-vector blocks of its main loop (oracle/ref_seq_harness.cpp),
      and achstemp from its own reduce_achstemp, on seeded inputs
      (workload.gpp_random).

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "fortkernels-_gb300"))
sys.path.insert(0, str(ROOT))

import workload as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

CONST_SHAPES = [(16, 2, 1024, 8), (32, 4, 2048, 10), (64, 1, 4096, 16), (128, 2, 8192, 20)]
FLAGOCC_CASES = {
    # name: (number_bands, ncouls, ngpown, seed, stress)
    "random_a": (3, 512, 32, 7, False),
    "random_b": (2, 999, 17, 21, False),
    "stress_a": (3, 512, 32, 8, True),
}


def closed_form(nb, nvband, ncouls, npg):
    ng = ncouls // npg
    wt = 0.5 + 0.5j
    wx = W.wx_frequencies()
    delw = wt * np.conj(wx - wt) / np.abs(wx - wt) ** 2
    ach = nb * ng * ncouls * 0.5 * 0.5 * delw * (0.5 + 0.5j)
    asx = nvband * ng * ncouls * 0.5 * (wt ** 2 * (0.5 + 0.5j) / wx ** 2)
    return ach, asx


def igp_map(prob):
    out = []
    for ind in prob.inv_igp_index:
        out.append(prob.ncouls - 1 if ind == prob.ncouls else int(prob.indinv[ind]))
    return np.array(out, dtype=np.int32)


FF_CONST_SHAPES = [(4, 2, 512, 32, 6, 5), (12, 3, 1000, 50, 8, 4), (20, 1, 777, 40, 12, 3)]
FF_RANDOM_CASES = {
    # name: (number_bands, nvband, ncouls, ngpown, nfreq, nfreqeval, seed, freqevalmin)
    "ff_random_a": (12, 2, 300, 20, 8, 4, 7, 0.3),
    "ff_random_b": (9, 3, 257, 13, 10, 3, 8, 0.7),
}


def ff_main():
    const = []
    for shape in FF_CONST_SHAPES:
        out = O.run_reference_ff_binary(*shape, threads=4)
        const.append({"shape": list(shape), **{k: [v.real, v.imag] for k, v in out.items()}})
        print(shape, out)
    rand = []
    for name, (nb, nv, nc, ng, nf, nfe, seed, fmin) in FF_RANDOM_CASES.items():
        p = W.ff_sigma_random(nb, nv, nc, ng, nf, nfe, seed)
        p.freqevalmin = fmin
        q = W.FFSigmaProblem(**p.__dict__)
        q.I_epsR = p.I_epsR.copy()
        q.I_epsR[1] = p.I_epsR[0]
        achs, _, _ = O.reference_ff_kernels(q, fmin - p.freqevalstep)
        _, asx, cor = O.reference_ff_kernels(p, fmin - p.freqevalstep)
        rand.append({"name": name, "args": [nb, nv, nc, ng, nf, nfe, seed], "freqevalmin": fmin,
                     "achsDtemp": [achs.real, achs.imag],
                     "asxDtemp_iw0": [[z.real, z.imag] for z in asx],
                     "achDtemp_cor_iw0": [[z.real, z.imag] for z in cor]})
        print(name, achs, asx[0], cor[0])
    (HERE / "ff_sigma_reference.json").write_text(json.dumps({
        "source": "FFKer_cori/ffKernel.cpp, unmodified, g++ -O3 -fopenmp -std=c++11: driver stdout "
                  "(6 decimals) on its constant fill; its kernels on seeded inputs",
        "constant_fill": const, "random": rand}, indent=1))


REAL_CONST_SHAPES = [(16, 2, 1024, 8), (32, 4, 2048, 16), (9, 1, 999, 9)]
REAL_FLAGOCC_CASES = {"real_a": (3, 300, 17, 5), "real_b": (2, 777, 33, 6)}


def real_main():
    runs = []
    for shape in REAL_CONST_SHAPES:
        ach = O.run_reference_real_binary(*shape, threads=4)
        runs.append({"shape": list(shape), "achtemp": [float(v) for v in ach]})
        print(shape, ach)
    (HERE / "gpp_real_reference.json").write_text(json.dumps({
        "source": "gppKer_real.cpp, unmodified, g++ -O3 -fopenmp -std=c++11; stdout achtemp (15 digits)",
        "runs": runs}, indent=1))
    for name, (nb, nc, ng, seed) in REAL_FLAGOCC_CASES.items():
        prob = W.gpp_real_random(nb, nb, nc, ng, seed)
        ssx, sch = O.reference_real_flagocc_columns(prob, igp_map(prob))
        np.savez_compressed(HERE / f"gpp_real_flagocc_{name}.npz", ssx=ssx, sch=sch,
                            meta=np.array([nb, nc, ng, seed]))
        print(name, np.abs(sch).max(), np.abs(ssx).max())


HALF_CONST_SHAPES = [(16, 2, 512, 4), (16, 0, 512, 4), (8, 8, 1024, 8), (24, 3, 1536, 3),
                     (32, 2, 2048, 16), (64, 4, 4096, 8)]
HALF_CASES = {
    # name: (number_bands, nvband, ncouls, ngpown, seed, stress); ncouls 1536 with
    # ngpown 33 puts igp on 512 and 1024 (the unpaired igp term of the blocked loop)
    "half_a": (6, 2, 1100, 40, 7, False),
    "half_b": (5, 3, 1536, 33, 8, False),
    "half_c": (4, 1, 1536, 33, 9, True),
}


def half_main():
    runs = []
    for shape in HALF_CONST_SHAPES:
        ach, secs, _ = O.run_reference_seq_binary(*shape, gppsum=1)
        runs.append({"shape": list(shape), "gppsum": 1, "achtemp": [[z.real, z.imag] for z in ach]})
        print(shape, ach, f"{secs:.2f}s")
    (HERE / "gpp_halfsum_reference.json").write_text(json.dumps({
        "source": "gppKerSeq.cpp, unmodified, g++ -O3 -fopenmp -std=c++14, argv gppsum = 1; "
                  "stdout achtemp (15 digits)",
        "runs": runs}, indent=1))
    for name, (nb, nvb, nc, ng, seed, stress) in HALF_CASES.items():
        prob = W.gpp_random(nb, nvb, nc, ng, seed, stress=stress)
        sch, ssx = O.reference_seq_columns(prob, igp_map(prob))
        stat = O.reference_seq_achstemp(prob)
        np.savez_compressed(HERE / f"gpp_halfsum_{name}.npz", sch=sch, ssx=ssx,
                            achstemp=np.array([stat]), meta=np.array([nb, nvb, nc, ng, seed, int(stress)]))
        print(name, np.abs(sch).max(), np.abs(ssx).max(), stat)


def main():
    if O.reference_lib() is None:
        sys.exit("reference checkout not found; set REFERENCE_ROOT")
    rows = []
    for shape in CONST_SHAPES:
        for threads in (1, 4):
            ach, secs, _ = O.run_reference_binary(*shape, threads=threads)
            exact, exact_asx = closed_form(*shape)
            rows.append({
                "shape": list(shape), "omp_threads": threads,
                "achtemp": [[z.real, z.imag] for z in ach],
                "closed_form_achtemp": [[z.real, z.imag] for z in exact],
                "closed_form_asxtemp": [[z.real, z.imag] for z in exact_asx],
            })
            print(shape, threads, ach)
    (HERE / "gpp_reference_constfill.json").write_text(json.dumps({
        "source": "BGW-Kernels/gppKer.cpp, unmodified, g++ -O3 -fopenmp -std=c++11; stdout achtemp (15 digits)",
        "runs": rows}, indent=1))

    for name, (nb, nc, ng, seed, stress) in FLAGOCC_CASES.items():
        prob = W.gpp_random(nb, nb, nc, ng, seed, stress=stress)
        ssx, sch = O.reference_flagocc_columns(prob, igp_map(prob))
        np.savez_compressed(HERE / f"gpp_flagocc_{name}.npz", ssx=ssx, sch=sch,
                            meta=np.array([nb, nc, ng, seed, int(stress)]))
        print(name, np.abs(sch).max(), np.abs(ssx).max())


if __name__ == "__main__":
    main()
    ff_main()
    real_main()
    half_main()
