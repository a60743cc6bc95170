"""The split-BF16 contraction's work entries (host code of ff_ozaki.cu):
every K' tile that a 128-row block may hold nonzero values in is covered by
exactly one entry and no other tile is, for the production shapes, the
half-sum triangle and 3000 random shapes with random per-row K limits.  The
check program links the library's objects and runs on the CPU."""
import pathlib
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_work_entries_cover_exactly_the_nonzero_tiles(tmp_path):
    import build as B
    B.build()
    obj = B.BUILD / "ff_ozaki.o"
    assert obj.exists()
    exe = tmp_path / "work_entries_check"
    cmd = [B.nvcc(), *B.ARCH, *B.NVCC_FLAGS, str(ROOT / "tests" / "csrc" / "work_entries_check.cu"),
           str(obj), "-o", str(exe), "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "cannot find -lcuda" in r.stderr:
        pytest.skip("no libcuda to link against")
    assert r.returncode == 0, r.stderr[-2000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert " 0 bad" in run.stdout
