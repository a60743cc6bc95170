"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker; the product library never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import re
import subprocess
import resource

import numpy as np

from . import build as _build

_lib = None
_port = None
_ref = None
_P, _I, _D = C.c_void_p, C.c_int, C.c_double

_GPP_ARGS = [_I, _I, _I, _I, _I, _I, _P, _P, _I, _P, _I, _D, _P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I]


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        l = C.CDLL(str(path))
        l.oracle_gpp.argtypes = _GPP_ARGS
        l.oracle_gpp_port.argtypes = _GPP_ARGS
        l.oracle_gpp_columns.argtypes = [_I, _I, _I, _I, _P, _P, _I, _P, _I, _P, _P, _P, _P, _P, _P,
                                         _I, _I, _I]
        l.oracle_ff_schdt.argtypes = [_I, _I, _I, _I, _P, _P, _P, _P, _P, _I, _P, _P, _P, _I]
        l.oracle_ff_sigma.argtypes = [_I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                      _D, _D, _D, _D, _P, _P, _P, _P, _P, _P, _P, _I]
        l.oracle_gpp_real.argtypes = [_I, _I, _I, _I, _P, _P, _I, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _I]
        l.oracle_gpp_achstemp.argtypes = [_I, _I, _I, _P, _P, _I, _P, _P, _P, _P, _P, _P, _I]
        l.oracle_gpp_abs2.argtypes = [_I, _I, _I, _I, _P, _P, _I, _P, _I, _D, _P, _P, _P, _P, _P, _P, _P,
                                      _I, _I, _I]
        _lib = l
    return _lib


def port_lib():
    """The same restatement built with the reference's -O3 flags (CPU timing)."""
    global _port
    if _port is None:
        l = C.CDLL(str(_build.build_port()))
        l.oracle_gpp_port.argtypes = _GPP_ARGS
        _port = l
    return _port


def _p(a):
    return None if a is None else a.ctypes.data


class OracleError(RuntimeError):
    pass


def _prep(prob):
    c = lambda a: np.ascontiguousarray(a, dtype=np.complex128)
    return (np.ascontiguousarray(prob.inv_igp_index, dtype=np.int32),
            np.ascontiguousarray(prob.indinv, dtype=np.int32),
            np.ascontiguousarray(prob.wx_array, dtype=np.float64),
            c(prob.aqsmtemp), c(prob.aqsntemp), c(prob.I_eps_array), c(prob.wtilde_array),
            np.ascontiguousarray(prob.vcoul, dtype=np.float64))


def gpp(prob, band_begin=0, band_end=None, nthreads=0, port=False, wx_band_stride=0):
    """Compensated oracle (or, port=True, the reference-order port) on a
    workload.GppProblem.  Returns (achtemp, asxtemp, acht_n1_loc) where
    acht_n1_loc holds zeros outside [band_begin, band_end)."""
    if band_end is None:
        band_end = prob.number_bands
    inv, indinv, wx, aqsm, aqsn, ieps, wt, vcoul = _prep(prob)
    ach = np.zeros(3, np.complex128)
    asx = np.zeros(3, np.complex128)
    n1 = np.zeros(prob.number_bands, np.complex128)
    fn = port_lib().oracle_gpp_port if port else lib().oracle_gpp
    st = fn(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, prob.nstart, prob.nend,
            _p(inv), _p(indinv), len(indinv), _p(wx), wx_band_stride, prob.occ, _p(aqsm), _p(aqsn),
            _p(ieps), _p(wt), _p(vcoul), _p(ach), _p(asx), _p(n1), band_begin, band_end, nthreads)
    if st != 0:
        raise OracleError(f"oracle_gpp status {st}")
    return ach, asx, n1


def gpp_columns(prob, band_begin=0, band_end=None, nthreads=0, wx_band_stride=0):
    """Per-(band, column, frequency) sch_array (0.5*scht) and ssx_array sums."""
    if band_end is None:
        band_end = prob.number_bands
    inv, indinv, wx, aqsm, aqsn, ieps, wt, _ = _prep(prob)
    nbr = band_end - band_begin
    sch = np.zeros((nbr, prob.ngpown, 3), np.complex128)
    ssx = np.zeros((nbr, prob.ngpown, 3), np.complex128)
    st = lib().oracle_gpp_columns(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, _p(inv),
                                  _p(indinv), len(indinv), _p(wx), wx_band_stride, _p(aqsm),
                                  _p(aqsn), _p(ieps), _p(wt), _p(sch), _p(ssx), band_begin,
                                  band_end, nthreads)
    if st != 0:
        raise OracleError(f"oracle_gpp_columns status {st}")
    return sch, ssx


def gpp_abs2(prob, band_begin=0, band_end=None, nthreads=0, wx_band_stride=0):
    """Sum of squared term magnitudes per output over bands [band_begin,
    band_end): (ach_abs2[3], asx_abs2[3])."""
    if band_end is None:
        band_end = prob.number_bands
    inv, indinv, wx, aqsm, aqsn, ieps, wt, vcoul = _prep(prob)
    a = np.zeros(3)
    x = np.zeros(3)
    st = lib().oracle_gpp_abs2(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, _p(inv),
                               _p(indinv), len(indinv), _p(wx), wx_band_stride, prob.occ, _p(aqsm),
                               _p(aqsn), _p(ieps), _p(wt), _p(vcoul), _p(a), _p(x), band_begin,
                               band_end, nthreads)
    if st != 0:
        raise OracleError(f"oracle_gpp_abs2 status {st}")
    return a, x


def gpp_achstemp(prob, nthreads=0):
    """Static remainder (Fortran formula): (achstemp, achstemp_n1[number_bands])."""
    inv, indinv, _, aqsm, aqsn, ieps, _, vcoul = _prep(prob)
    out = np.zeros(1, np.complex128)
    n1 = np.zeros(prob.number_bands, np.complex128)
    st = lib().oracle_gpp_achstemp(prob.number_bands, prob.ncouls, prob.ngpown, _p(inv), _p(indinv),
                                   len(indinv), _p(aqsm), _p(aqsn), _p(ieps), _p(vcoul), _p(out), _p(n1),
                                   nthreads)
    if st != 0:
        raise OracleError(f"oracle_gpp_achstemp status {st}")
    return out[0], n1


def ff_schdt(prob, entries=None, nthreads=0):
    """schDt[n1][ifreq] for the (n1, ifreq) pairs in `entries` (default all)."""
    if entries is None:
        entries = [(n, f) for n in range(prob.number_bands) for f in range(prob.nfreq)]
    en = np.ascontiguousarray([e[0] for e in entries], dtype=np.int32)
    ef = np.ascontiguousarray([e[1] for e in entries], dtype=np.int32)
    out = np.zeros(len(entries), np.complex128)
    c = lambda a: np.ascontiguousarray(a, dtype=np.complex128)
    inv = np.ascontiguousarray(prob.inv_igp_index, dtype=np.int32)
    indinv = np.ascontiguousarray(prob.indinv, dtype=np.int32)
    epsr, aqsn, aqsm = c(prob.I_epsR), c(prob.aqsntemp), c(prob.aqsmtemp)
    st = lib().oracle_ff_schdt(prob.number_bands, prob.ncouls, prob.ngpown, prob.nfreq, _p(inv),
                               _p(indinv), _p(epsr), _p(aqsn), _p(aqsm), len(entries), _p(en),
                               _p(ef), _p(out), nthreads)
    if st != 0:
        raise OracleError(f"oracle_ff_schdt status {st}")
    return out


# ---------------------------------------------------------------- the reference itself
def reference_lib():
    """The reference's flagOCC_solver through oracle/ref_harness.cpp (None when
    the reference checkout is absent)."""
    global _ref
    if _ref is None:
        if not _build.build_reference():
            return None
        l = C.CDLL(str(_build.REF_LIB))
        l.ref_flagocc_columns.argtypes = [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]
        l.ref_main.argtypes = [_I, _I, _I, _I]
        _ref = l
    return _ref


def reference_flagocc_columns(prob, igp_of):
    """(ssx_array, sch_array) per (band, column, frequency) from the reference's
    own flagOCC_solver on the problem's arrays."""
    l = reference_lib()
    if l is None:
        return None
    nb, ng = prob.number_bands, prob.ngpown
    arrs = [np.array(a, dtype=np.complex128, order="C", copy=True)
            for a in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array)]
    ssx = np.zeros((nb, ng, 3), np.complex128)
    sch = np.zeros((nb, ng, 3), np.complex128)
    igp = np.ascontiguousarray(igp_of, dtype=np.int32)
    wx = np.ascontiguousarray(prob.wx_array, dtype=np.float64)
    l.ref_flagocc_columns(nb, prob.ncouls, ng, _p(igp), _p(wx), *[_p(a) for a in arrs], _p(ssx), _p(sch))
    return ssx, sch


_ACH = re.compile(r"achtemp\[(\d+)\] = \(([-+0-9.eE]+),([-+0-9.eE]+)\)")
_TIME = re.compile(r"Chrono Time Taken \*+= ([0-9.eE+-]+) secs")


def run_reference_binary(number_bands, nvband, ncouls, nodes_per_group, threads=None, timeout=900):
    """Runs the unmodified reference driver; returns (achtemp[3], seconds, stdout)."""
    if not _build.build_reference():
        return None
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    env.setdefault("OMP_STACKSIZE", "64M")

    def _unlimit_stack():
        try:
            resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))
        except (ValueError, OSError):
            pass

    r = subprocess.run([str(_build.REF_BIN), str(number_bands), str(nvband), str(ncouls),
                        str(nodes_per_group)], capture_output=True, text=True, env=env,
                       timeout=timeout, preexec_fn=_unlimit_stack)
    ach = np.zeros(3, np.complex128)
    for m in _ACH.finditer(r.stdout):
        ach[int(m.group(1))] = complex(float(m.group(2)), float(m.group(3)))
    t = _TIME.search(r.stdout)
    return ach, (float(t.group(1)) if t else float("nan")), r.stdout


_ffref = None


def reference_ff_lib():
    """The reference's FF kernels through oracle/ff_ref_harness.cpp (None when
    the reference checkout is absent)."""
    global _ffref
    if _ffref is None:
        if not _build.build_reference() or not _build.FF_REF_LIB.exists():
            return None
        l = C.CDLL(str(_build.FF_REF_LIB))
        l.ref_ff_kernels.argtypes = [_I] * 6 + [_D] * 3 + [_P] * 12
        _ffref = l
    return _ffref


def reference_ff_kernels(prob, freqevalmin):
    """(achsDtemp, asxDtemp[nfreqeval], achDtemp_cor[nfreqeval]) from the
    reference's own achsDtemp_Kernel / asxDtemp_Kernel / achDtemp_cor_Kernel
    (FFKer_cori/ffKernel.cpp:107-245) on the problem's arrays."""
    l = reference_ff_lib()
    if l is None:
        return None
    c = lambda a: np.array(a, dtype=np.complex128, order="C", copy=True)
    i32 = lambda a: np.array(a, dtype=np.int32, order="C", copy=True)
    f = lambda a: np.array(a, dtype=np.float64, order="C", copy=True)
    p = prob
    arrs = [i32(p.inv_igp_index), i32(p.indinv), c(p.aqsmtemp), c(p.aqsntemp), c(p.I_epsR), c(p.I_epsA),
            f(p.vcoul), f(p.ekq), f(p.dFreqGrid)]
    achs = np.zeros(1, np.complex128)
    asx = np.zeros(p.nfreqeval, np.complex128)
    cor = np.zeros(p.nfreqeval, np.complex128)
    l.ref_ff_kernels(p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nfreq, p.nfreqeval, freqevalmin,
                     p.freqevalstep, p.occ, *[_p(a) for a in arrs], _p(achs), _p(asx), _p(cor))
    return achs[0], asx, cor


_FFOUT = re.compile(r"(achsDtemp|asxDtemp|achDtemp_cor) = \( *([-+0-9.eE]+), *([-+0-9.eE]+)\)")


def run_reference_ff_binary(number_bands, nvband, ncouls, ngpown, nfreq, nfreqeval, threads=None,
                            timeout=600):
    """Runs the unmodified FFKer_cori/ffKernel.cpp driver (its constant fill);
    returns its printed achsDtemp, asxDtemp[0], achDtemp_cor[0]."""
    if not _build.build_reference() or not _build.FF_REF_BIN.exists():
        return None
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    r = subprocess.run([str(_build.FF_REF_BIN), str(number_bands), str(nvband), str(ncouls), str(ngpown),
                        str(nfreq), str(nfreqeval)], capture_output=True, text=True, env=env,
                       timeout=timeout)
    return {m.group(1): complex(float(m.group(2)), float(m.group(3))) for m in _FFOUT.finditer(r.stdout)}


def ff_sigma(prob, schdt=None, nthreads=0):
    """Full-frequency sigma (Fortran band loop) on a workload.FFSigmaProblem.
    schdt: complex [number_bands][nfreq] (default zeros, as the live Fortran
    leaves it).  Returns dict(achsDtemp, asxDtemp, achDtemp, achDtemp_cor,
    achDtemp_corb, ach2Dtemp)."""
    c = lambda a: np.ascontiguousarray(a, dtype=np.complex128)
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    p = prob
    if schdt is None:
        schdt = np.zeros((p.number_bands, p.nfreq), np.complex128)
    args = [i32(p.inv_igp_index), i32(p.indinv), c(p.aqsmtemp), c(p.aqsntemp), c(p.I_epsR), c(p.I_epsA),
            f(p.vcoul), f(p.ekq), f(p.dFreqGrid), c(p.dFreqBrd), f(p.pref)]
    sd = c(schdt)
    out = {k: np.zeros(1 if k == "achsDtemp" else p.nfreqeval, np.complex128)
           for k in ("achsDtemp", "asxDtemp", "achDtemp", "achDtemp_cor", "achDtemp_corb", "ach2Dtemp")}
    st = lib().oracle_ff_sigma(p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nfreq, p.nfreqeval,
                               *[_p(a) for a in args], p.pref_zb, p.freqevalmin, p.freqevalstep, p.occ,
                               _p(sd), *[_p(out[k]) for k in ("achsDtemp", "asxDtemp", "achDtemp",
                                                               "achDtemp_cor", "achDtemp_corb",
                                                               "ach2Dtemp")], nthreads)
    if st != 0:
        raise OracleError(f"oracle_ff_sigma status {st}")
    out["achsDtemp"] = out["achsDtemp"][0]
    return out


def gpp_real(prob, nthreads=0):
    """Real-valued GPP (gppKer_real.cpp semantics): (achtemp[3], asxtemp[3],
    acht_n1_loc[nb]) float64."""
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    p = prob
    inv, ind = i32(p.inv_igp_index), i32(p.indinv)
    arrs = [f(p.wx_array)]
    ach, asx, n1 = np.zeros(3), np.zeros(3), np.zeros(p.number_bands)
    data = [f(p.aqsmtemp), f(p.aqsntemp), f(p.I_eps_array), f(p.wtilde_array), f(p.vcoul)]
    st = lib().oracle_gpp_real(p.number_bands, p.nvband, p.ncouls, p.ngpown, _p(inv), _p(ind), len(ind),
                               _p(arrs[0]), p.occ, *[_p(a) for a in data], _p(ach), _p(asx), _p(n1), nthreads)
    if st != 0:
        raise OracleError(f"oracle_gpp_real status {st}")
    return ach, asx, n1


_realref = None


def reference_real_flagocc_columns(prob, igp_of):
    """(ssx_array, sch_array) per (band, column, frequency) from the real
    mini-app's own flagOCC_solver (gppKer_real.cpp:124-155)."""
    global _realref
    if _realref is None:
        if not _build.build_reference() or not _build.REAL_REF_LIB.exists():
            return None
        l = C.CDLL(str(_build.REAL_REF_LIB))
        l.ref_real_flagocc_columns.argtypes = [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]
        _realref = l
    nb, ng = prob.number_bands, prob.ngpown
    arrs = [np.array(a, dtype=np.float64, order="C", copy=True)
            for a in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array)]
    ssx = np.zeros((nb, ng, 3))
    sch = np.zeros((nb, ng, 3))
    igp = np.ascontiguousarray(igp_of, dtype=np.int32)
    wx = np.ascontiguousarray(prob.wx_array, dtype=np.float64)
    _realref.ref_real_flagocc_columns(nb, prob.ncouls, ng, _p(igp), _p(wx), *[_p(a) for a in arrs], _p(ssx),
                                      _p(sch))
    return ssx, sch


def run_reference_real_binary(number_bands, nvband, ncouls, nodes_per_group, threads=None, timeout=600):
    """Runs the unmodified gppKer_real.cpp driver (its constant fill); returns achtemp[3]."""
    if not _build.build_reference() or not _build.REAL_REF_BIN.exists():
        return None
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    env.setdefault("OMP_STACKSIZE", "64M")
    r = subprocess.run([str(_build.REAL_REF_BIN), str(number_bands), str(nvband), str(ncouls),
                        str(nodes_per_group)], capture_output=True, text=True, env=env, timeout=timeout)
    out = np.zeros(3)
    for m in re.finditer(r"achtemp\[(\d+)\] = ([-+0-9.eE]+)", r.stdout):
        out[int(m.group(1))] = float(m.group(2))
    return out


def gpp_halfsum(prob, nthreads=0, columns=False, band_begin=0, band_end=None):
    """gppsum = 1 ("half sum") GPP of gppKerSeq.cpp on a GppProblem in
    band-major layout.  Returns (achtemp[3], asxtemp[3], acht_n1_loc[nb],
    achstemp) complex128, plus (col_sch, col_ssx) [nb][ng][3] with
    columns=True; sums over bands [band_begin, band_end) (all by default)."""
    l = lib()
    if not hasattr(l, "_halfsum_ready"):
        l.oracle_gpp_halfsum.argtypes = [_I, _I, _I, _I, _P, _P, _I, _P, _D, _P, _P, _P, _P, _P, _P, _P,
                                         _P, _P, _P, _P, _I, _I, _I]
        l._halfsum_ready = True
    band_end = prob.number_bands if band_end is None else band_end
    inv, indinv, wx, aqsm, aqsn, ieps, wt, vcoul = _prep(prob)
    nb, ng = prob.number_bands, prob.ngpown
    ach, asx = np.zeros(3, np.complex128), np.zeros(3, np.complex128)
    n1, stat = np.zeros(nb, np.complex128), np.zeros(1, np.complex128)
    cs = np.zeros((nb, ng, 3), np.complex128) if columns else None
    cx = np.zeros((nb, ng, 3), np.complex128) if columns else None
    st = l.oracle_gpp_halfsum(nb, prob.nvband, prob.ncouls, ng, _p(inv), _p(indinv), len(indinv), _p(wx[:3]),
                              float(getattr(prob, "occ", 1.0)), _p(aqsm), _p(aqsn), _p(ieps), _p(wt),
                              _p(vcoul), _p(ach), _p(asx), _p(n1), _p(stat), _p(cs), _p(cx), nthreads,
                              band_begin, band_end)
    if st != 0:
        raise OracleError(f"oracle_gpp_halfsum status {st}")
    out = (ach, asx, n1, stat[0])
    return out + (cs, cx) if columns else out


_seqref = None


def reference_seq_lib():
    """gppKerSeq.cpp's own solvers through oracle/ref_seq_harness.cpp (None
    when the reference checkout is absent)."""
    global _seqref
    if _seqref is None:
        if not _build.build_reference() or not _build.SEQ_REF_LIB.exists():
            return None
        l = C.CDLL(str(_build.SEQ_REF_LIB))
        l.ref_seq_columns.argtypes = [_I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]
        l.ref_seq_achstemp.argtypes = [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P]
        l.ref_seq_main.argtypes = [_I, _I, _I, _I, _I]
        _seqref = l
    return _seqref


def reference_seq_columns(prob, igp_of):
    """(sch_array, ssx_array) per (band, column, frequency) from gppKerSeq.cpp's
    own gppsum = 1 solvers, driven as its main loop drives them."""
    l = reference_seq_lib()
    if l is None:
        return None
    nb, ng = prob.number_bands, prob.ngpown
    _, _, wx, aqsm, aqsn, ieps, wt, _ = _prep(prob)
    sch = np.zeros((nb, ng, 3), np.complex128)
    ssx = np.zeros((nb, ng, 3), np.complex128)
    igp = np.ascontiguousarray(igp_of, dtype=np.int32)
    l.ref_seq_columns(nb, prob.nvband, prob.ncouls, ng, _p(igp), _p(wx[:3]), _p(aqsm), _p(aqsn), _p(ieps),
                      _p(wt), _p(sch), _p(ssx))
    return sch, ssx


def reference_seq_achstemp(prob):
    """achstemp after gppKerSeq.cpp's own reduce_achstemp (gppsum = 1) over every band."""
    l = reference_seq_lib()
    if l is None:
        return None
    inv, indinv, _, aqsm, aqsn, ieps, _, vcoul = _prep(prob)
    inv, indinv, vcoul = inv.copy(), indinv.copy(), vcoul.copy()
    out = np.zeros(1, np.complex128)
    l.ref_seq_achstemp(prob.number_bands, prob.ncouls, prob.ngpown, _p(inv), _p(indinv), _p(aqsm), _p(aqsn),
                       _p(ieps), _p(vcoul), _p(out))
    return out[0]


def run_reference_seq_binary(number_bands, nvband, ncouls, nodes_per_group, gppsum=1, timeout=900):
    """Runs the unmodified gppKerSeq.cpp driver (its constant fill); returns
    (achtemp[3], seconds, stdout)."""
    if not _build.build_reference() or not _build.SEQ_REF_BIN.exists():
        return None

    def _unlimit_stack():
        try:
            resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))
        except (ValueError, OSError):
            pass

    r = subprocess.run([str(_build.SEQ_REF_BIN), str(number_bands), str(nvband), str(ncouls),
                        str(nodes_per_group), str(gppsum)], capture_output=True, text=True,
                       timeout=timeout, preexec_fn=_unlimit_stack)
    ach = np.zeros(3, np.complex128)
    for m in _ACH.finditer(r.stdout):
        ach[int(m.group(1))] = complex(float(m.group(2)), float(m.group(3)))
    t = re.search(r"Time Taken \*+= ([0-9.eE+-]+)", r.stdout)
    return ach, (float(t.group(1)) if t else float("nan")), r.stdout
