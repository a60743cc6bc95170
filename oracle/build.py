"""Build recipe of the CPU oracle (test infrastructure only).

  oracle/_build/liboracle.so  <- oracle/gpp_oracle.cpp + oracle/gpp_halfsum_oracle.cpp
                                 (the C++ restatements)
  oracle/_ref/gppKer          <- BGW-Kernels/gppKer.cpp of the reference, unmodified
  oracle/_ref/libgppref.so    <- the same file (main renamed by -D) + oracle/ref_harness.cpp
  oracle/_ref/ffKernel        <- FFKer_cori/ffKernel.cpp of the reference, unmodified
  oracle/_ref/libffref.so     <- the same file (main renamed by -D) + oracle/ff_ref_harness.cpp
  oracle/_ref/gppKer_real     <- gppKer_real.cpp of the reference, unmodified
  oracle/_ref/libgpprealref.so <- the same file (main renamed by -D) + oracle/ref_real_harness.cpp
  oracle/_ref/gppKerSeq       <- gppKerSeq.cpp of the reference, unmodified (the gppsum = 1 driver)
  oracle/_ref/libgppseqref.so <- the same file (main renamed by -D) + oracle/ref_seq_harness.cpp

The oracle/_ref products are built only where the reference checkout is
present (REFERENCE_ROOT, default: a checkout named `reference` beside this
repository); they are compiled from the
reference's own source file in place and nothing of it is copied.
"""
from __future__ import annotations

import os
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_LIB = BUILD / "liboracle.so"
PORT_LIB = BUILD / "libport.so"
REF_BIN = REF_OUT / "gppKer"
REF_LIB = REF_OUT / "libgppref.so"
REFERENCE_ROOT = pathlib.Path(os.environ.get("REFERENCE_ROOT", HERE.parents[1] / "reference"))
REF_SRC = REFERENCE_ROOT / "BGW-Kernels" / "gppKer.cpp"
FF_REF_DIR = REFERENCE_ROOT / "FFKer_cori"
FF_REF_SRC = FF_REF_DIR / "ffKernel.cpp"
FF_REF_BIN = REF_OUT / "ffKernel"
FF_REF_LIB = REF_OUT / "libffref.so"
REAL_REF_SRC = REFERENCE_ROOT / "gppKer_real.cpp"
REAL_REF_BIN = REF_OUT / "gppKer_real"
REAL_REF_LIB = REF_OUT / "libgpprealref.so"
SEQ_REF_SRC = REFERENCE_ROOT / "gppKerSeq.cpp"
SEQ_REF_BIN = REF_OUT / "gppKerSeq"
SEQ_REF_LIB = REF_OUT / "libgppseqref.so"
ORACLE_SRCS = ("gpp_oracle.cpp", "gpp_halfsum_oracle.cpp")

ORACLE_FLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]
# the timing build of the same file: the reference's own optimisation flags
PORT_FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared"]
REF_FLAGS = ["-O3", "-std=c++11", "-fopenmp"]
# gppKerSeq.cpp writes `0.0 + 0.0i` (:121), a C++14 complex literal
SEQ_REF_FLAGS = ["-O3", "-std=c++14", "-fopenmp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def _newer(target: pathlib.Path, *deps: pathlib.Path) -> bool:
    return target.exists() and all(target.stat().st_mtime >= d.stat().st_mtime for d in deps)


def build_oracle() -> pathlib.Path:
    srcs = [HERE / f for f in ORACLE_SRCS]
    if _newer(ORACLE_LIB, *srcs):
        return ORACLE_LIB
    BUILD.mkdir(exist_ok=True)
    _run(["g++", *ORACLE_FLAGS, *map(str, srcs), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def build_port() -> pathlib.Path:
    """The oracle sources built with -O3 like the reference, for CPU timing."""
    srcs = [HERE / f for f in ORACLE_SRCS]
    if _newer(PORT_LIB, *srcs):
        return PORT_LIB
    BUILD.mkdir(exist_ok=True)
    _run(["g++", *PORT_FLAGS, *map(str, srcs), "-o", str(PORT_LIB)])
    return PORT_LIB


def reference_available() -> bool:
    return REF_SRC.exists()


def build_reference() -> bool:
    """Builds oracle/_ref from the reference source; False when it is absent."""
    if not reference_available():
        return False
    REF_OUT.mkdir(exist_ok=True)
    if not _newer(REF_BIN, REF_SRC):
        _run(["g++", *REF_FLAGS, str(REF_SRC), "-o", str(REF_BIN)])
    harness = HERE / "ref_harness.cpp"
    if not _newer(REF_LIB, REF_SRC, harness):
        _run(["g++", *REF_FLAGS, "-fPIC", "-shared", "-Dmain=gppker_reference_main",
              str(REF_SRC), str(harness), "-o", str(REF_LIB)])
    if FF_REF_SRC.exists():
        inc = ["-I", str(FF_REF_DIR)]
        if not _newer(FF_REF_BIN, FF_REF_SRC):
            _run(["g++", *REF_FLAGS, *inc, str(FF_REF_SRC), "-o", str(FF_REF_BIN)])
        ffh = HERE / "ff_ref_harness.cpp"
        if not _newer(FF_REF_LIB, FF_REF_SRC, ffh):
            _run(["g++", *REF_FLAGS, *inc, "-fPIC", "-shared", "-Dmain=ffker_reference_main",
                  str(FF_REF_SRC), str(ffh), "-o", str(FF_REF_LIB)])
    if REAL_REF_SRC.exists():
        if not _newer(REAL_REF_BIN, REAL_REF_SRC):
            _run(["g++", *REF_FLAGS, str(REAL_REF_SRC), "-o", str(REAL_REF_BIN)])
        rh = HERE / "ref_real_harness.cpp"
        if not _newer(REAL_REF_LIB, REAL_REF_SRC, rh):
            _run(["g++", *REF_FLAGS, "-fPIC", "-shared", "-Dmain=gppreal_reference_main",
                  str(REAL_REF_SRC), str(rh), "-o", str(REAL_REF_LIB)])
    if SEQ_REF_SRC.exists():
        if not _newer(SEQ_REF_BIN, SEQ_REF_SRC):
            _run(["g++", *SEQ_REF_FLAGS, str(SEQ_REF_SRC), "-o", str(SEQ_REF_BIN)])
        sh = HERE / "ref_seq_harness.cpp"
        if not _newer(SEQ_REF_LIB, SEQ_REF_SRC, sh):
            _run(["g++", *SEQ_REF_FLAGS, "-fPIC", "-shared", "-Dmain=gppseq_reference_main",
                  str(SEQ_REF_SRC), str(sh), "-o", str(SEQ_REF_LIB)])
    return True


if __name__ == "__main__":
    print(build_oracle())
    print(build_port())
    print("reference:", build_reference())
