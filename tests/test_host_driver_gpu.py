"""The C++ command-line driver (host/gppKer_gb300.cpp) against the
unmodified reference driver's output.

host/gppKer_gb300.cpp takes the reference CLI (<number_bands>
<number_valence_bands> <number_plane_waves> <nodes_per_group>,
BGW-Kernels/gppKer.cpp:164-176), builds the same constant fill
(:275-299) and prints achtemp with 15 digits as the reference does
(:441-446), computing through the sigma_gpp_fp64 C ABI.  Its printed values
are compared with the unmodified reference's printed values
(tests/golden/gpp_reference_constfill.json, made by make_golden.py from the
reference binary) and with the fill's closed form.

Tolerances: the closed form within 1e-12 relative (the FP64 bar); the
reference's printed values within 1e-12 plus that run's own deviation from
the closed form (its OpenMP partial sums deviate by up to 1.3e-12).
"""
import json
import pathlib
import re
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "gpp_reference_constfill.json"
_ACH = re.compile(r"achtemp\[(\d+)\] = \(([-+0-9.eE]+),([-+0-9.eE]+)\)")


def _run_driver(exe, shape):
    r = subprocess.run([str(exe), *map(str, shape)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = {int(m.group(1)): complex(float(m.group(2)), float(m.group(3))) for m in _ACH.finditer(r.stdout)}
    assert sorted(vals) == [0, 1, 2], r.stdout
    return np.array([vals[i] for i in range(3)])


def test_driver_matches_reference_stdout(sigma_lib):
    import build as B

    exe = B.build_host_driver()
    runs = json.loads(GOLDEN.read_text())["runs"]
    for shape in sorted({tuple(r["shape"]) for r in runs}):
        got = _run_driver(exe, shape)
        rows = [r for r in runs if tuple(r["shape"]) == shape]
        exact = np.array([complex(*z) for z in rows[0]["closed_form_achtemp"]])
        assert np.max(np.abs(got - exact) / np.abs(exact)) <= 1e-12, (shape, got, exact)
        for r in rows:
            ref = np.array([complex(*z) for z in r["achtemp"]])
            own = np.max(np.abs(ref - exact) / np.abs(exact))
            assert np.max(np.abs(got - ref) / np.abs(ref)) <= 1e-12 + own, (shape, r["omp_threads"])
