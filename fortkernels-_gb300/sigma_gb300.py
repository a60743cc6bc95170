"""ctypes binding of libsigma_gb300.so, the sigma GPP / FF C ABI (include/*.h).

The functions mirror the reference's calls: `gpp_fp64` / `gpp_mixed` take the
arrays BGW-Kernels/gppKer.cpp builds in main() and return achtemp, asxtemp and
acht_n1_loc as its loop nest :303-439 would leave them.  There is no CPU
fallback: loading fails with an exception when the library is missing or no
CUDA device is present, and every non-zero status raises SigmaError.
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libsigma_gb300.so"

OK = 0
PREC_FP64, PREC_MIXED, PREC_TENSOR = 0, 1, 2
FF_MODE_FP64, FF_MODE_OZAKI_BF16 = 0, 1

STATUS = {
    0: "ok", -1: "invalid shape", -2: "index out of range", -3: "allocation failed",
    -4: "CUDA error", -5: "device wait timed out", -6: "null pointer", -7: "no usable CUDA device",
    -8: "unsupported argument combination", -9: "workspace too small",
}


class SigmaError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: {STATUS.get(status, 'unknown')} ({status})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


_lib = None

_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_LL = C.c_longlong
_ULL = C.c_ulonglong

# name -> argtypes (restype int unless noted)
SIGNATURES = {
    "sigma_status_string": ([_I], C.c_char_p),
    "sigma_last_error_message": ([], C.c_char_p),
    "sigma_shutdown": ([], _I),
    "sigma_version": ([], C.c_char_p),
    "sigma_gpp_fp64": ([_I, _I, _I, _I, _I, _I, _P, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "sigma_gpp_mixed": ([_I, _I, _I, _I, _I, _I, _P, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "sigma_gpp_tensor": ([_I, _I, _I, _I, _I, _I, _P, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "sigma_gpp_mixed_checked": ([_I, _I, _I, _I, _I, _I, _P, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                 _P], _I),
    "sigma_gpp_plan_create": ([_P, _I, _I, _I, _I, _I, _I, _P, _P, _I, _I], _I),
    "sigma_gpp_execute": ([_P, _P, _I, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "sigma_gpp_plan_destroy": ([_P], _I),
    "sigma_gpp_plan_info": ([_P, _P, _P], _I),
    "sigma_gpp_plan_status": ([_P, _P], _I),
    "sigma_gpp_selftest_gate_timeout": ([_P, _P, _P, _P, _P, _P, _P, _I, _P], _I),
    "sigma_gpp_plan_set_timing": ([_P, _I], _I),
    "sigma_gpp_plan_timing": ([_P, _P, _P, _P, _P, _P], _I),
    "sigma_gpp_fp64_noalloc": ([_I, _I, _I, _I, _P, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "sigma_gpp_batch_create": ([_P, _I, _P, _I, _P], _I),
    "sigma_gpp_batch_create_tuned": ([_P, _I, _P, _I, _P, _I, _I], _I),
    "sigma_gpp_batch_execute": ([_P, _P], _I),
    "sigma_gpp_batch_launch_graph": ([_P, _P], _I),
    "sigma_gpp_batch_info": ([_P, _P, _P, _P], _I),
    "sigma_gpp_batch_status": ([_P, _P], _I),
    "sigma_gpp_batch_destroy": ([_P], _I),
    "sigma_gpp_batched": ([_I, _P, _I, _P], _I),
    "sigma_gpp_real_fp64": ([_I, _I, _I, _I, _I, _I, _P, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "sigma_gpp_real_plan_create": ([_P, _I, _I, _I, _I, _I, _I, _P, _P, _I], _I),
    "sigma_gpp_real_execute": ([_P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "sigma_gpp_real_plan_destroy": ([_P], _I),
    "sigma_gpp_halfsum_fp64": ([_I, _I, _I, _I, _I, _I, _P, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
                               _I),
    "sigma_gpp_halfsum_tensor": ([_I, _I, _I, _I, _I, _I, _P, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
                                 _I),
    "sigma_gpp_halfsum_plan_create": ([_P, _I, _I, _I, _I, _I, _I, _P, _P, _I, _I], _I),
    "sigma_gpp_halfsum_execute": ([_P, _P, _D] + [_P] * 10, _I),
    "sigma_gpp_halfsum_plan_destroy": ([_P], _I),
    "sigma_gpp_achstemp": ([_I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _I, _P], _I),
    "sigma_gpp_static_plan_create": ([_P, _I, _I, _I, _P, _P, _I], _I),
    "sigma_gpp_static_execute": ([_P, _P, _P, _P, _P, _P, _P, _P], _I),
    "sigma_ff_plan_bands": ([_P, _P], _I),
    "sigma_ff_sigma": ([_I] * 6 + [_P] * 11 + [_D] * 4 + [_P] * 7 + [_I, _P], _I),
    "sigma_ff_sigma_plan_create": ([_P, _I, _I, _I, _I, _I, _I, _P, _P, _I], _I),
    "sigma_ff_sigma_execute": ([_P] * 10 + [_D] * 4 + [_P, _P, _P], _I),
    "sigma_ff_sigma_plan_set_timing": ([_P, _I], _I),
    "sigma_ff_sigma_plan_timing": ([_P, _P, _P, _P], _I),
    "sigma_ff_sigma_plan_status": ([_P, _P], _I),
    "sigma_ff_sigma_plan_destroy": ([_P], _I),
    "sigma_ff_schdt": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _I, _P], _I),
    "sigma_ff_plan_create": ([_P, _I, _I, _I, _I, _P, _P, _I], _I),
    "sigma_ff_execute": ([_P, _P, _P, _P, _P, _P], _I),
    "sigma_ff_plan_destroy": ([_P], _I),
    "sigma_ff_plan_set_timing": ([_P, _I], _I),
    "sigma_ff_plan_timing": ([_P, _P, _P, _P, _P], _I),
    "sigma_ff_plan_status": ([_P, _P], _I),
    "sigma_fill_uniform": ([_P, _LL, _LL, _ULL, _ULL, _LL, _LL, _D, _D, _P], _I),
    "sigma_fill_stress": ([_P, _LL, _ULL, _ULL, _P, _I, _D, _D, _P], _I),
    "sigma_measure_fma_peaks": ([_P, _P, _P], _I),
    "sigma_eval_reciprocals": ([_P, _P, _LL, _P], _I),
    "sigma_eval_split": ([_P, _P, _LL, _P], _I),
    "sigma_eval_split_round": ([_P, _P, _LL, _P], _I),
}


def load(path: pathlib.Path | str | None = None):
    """Loads the CUDA library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("_sigma_build", PKG / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = C.CDLL(str(p))
    for name, (args, res) in SIGNATURES.items():
        if hasattr(lib, name):
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(SIGNATURES)


def _check(status: int, where: str):
    if status != OK:
        detail = ""
        if status == -4 and _lib is not None:
            detail = _lib.sigma_last_error_message().decode(errors="replace")
        raise SigmaError(status, where, detail)


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    # torch tensors (device or host)
    return a.data_ptr()


def _c128(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def gpp_host(prob, precision: int = PREC_FP64, stream: int = 0, want_n1: bool = True):
    """Runs the host-pointer drop-in on a workload.GppProblem; returns
    (achtemp[3], asxtemp[3], acht_n1_loc[nb]) as complex128 arrays."""
    lib = load()
    inv = np.ascontiguousarray(prob.inv_igp_index, dtype=np.int32)
    indinv = np.ascontiguousarray(prob.indinv, dtype=np.int32)
    wx = np.ascontiguousarray(prob.wx_array, dtype=np.float64)
    arrs = [_c128(prob.aqsmtemp), _c128(prob.aqsntemp), _c128(prob.I_eps_array), _c128(prob.wtilde_array)]
    vcoul = np.ascontiguousarray(prob.vcoul, dtype=np.float64)
    ach = np.zeros(3, np.complex128)
    asx = np.zeros(3, np.complex128)
    n1 = np.zeros(prob.number_bands, np.complex128) if want_n1 else None
    fn = {PREC_FP64: lib.sigma_gpp_fp64, PREC_MIXED: lib.sigma_gpp_mixed,
          PREC_TENSOR: lib.sigma_gpp_tensor}[precision]
    st = fn(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, prob.nstart, prob.nend,
            _ptr(inv), _ptr(indinv), _ptr(wx), prob.occ, *[_ptr(a) for a in arrs], _ptr(vcoul),
            _ptr(ach), _ptr(asx), _ptr(n1), stream)
    _check(st, fn.__name__)
    return ach, asx, n1


def gpp_real_host(prob, stream: int = 0, want_n1: bool = True):
    """Real-valued GPP host drop-in (sigma_gpp_real_fp64) on a
    workload.GppProblem with real arrays; returns (achtemp[3], asxtemp[3],
    acht_n1_loc[nb]) float64."""
    lib = load()
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    inv = np.ascontiguousarray(prob.inv_igp_index, dtype=np.int32)
    indinv = np.ascontiguousarray(prob.indinv, dtype=np.int32)
    arrs = [f(prob.wx_array), f(prob.aqsmtemp), f(prob.aqsntemp), f(prob.I_eps_array), f(prob.wtilde_array),
            f(prob.vcoul)]
    ach, asx = np.zeros(3), np.zeros(3)
    n1 = np.zeros(prob.number_bands) if want_n1 else None
    st = lib.sigma_gpp_real_fp64(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, prob.nstart,
                                 prob.nend, _ptr(inv), _ptr(indinv), _ptr(arrs[0]), prob.occ,
                                 *[_ptr(a) for a in arrs[1:]], _ptr(ach), _ptr(asx), _ptr(n1), stream)
    _check(st, "sigma_gpp_real_fp64")
    return ach, asx, n1


HALFSUM_STATIC, HALFSUM_GVEC_MAJOR, HALFSUM_TENSOR = 1, 2, 4


def gpp_halfsum_host(prob, stream: int = 0, want_n1: bool = True, want_static: bool = True,
                     tensor: bool = False):
    """gppsum = 1 host drop-in (sigma_gpp_halfsum_fp64, or with tensor=True
    sigma_gpp_halfsum_tensor) on a workload.GppProblem held band-major; the
    arrays are handed over in gppKerSeq.cpp's g-vector-major layout, as that
    driver stores them.  Returns (achtemp[3], asxtemp[3], acht_n1_loc[nb] or
    None, achstemp or None) complex128."""
    lib = load()
    inv = np.ascontiguousarray(prob.inv_igp_index, dtype=np.int32)
    indinv = np.ascontiguousarray(prob.indinv, dtype=np.int32)
    wx = np.ascontiguousarray(prob.wx_array[:3], dtype=np.float64)
    arrs = [_c128(np.asarray(a).T) for a in (prob.aqsmtemp, prob.aqsntemp, prob.I_eps_array, prob.wtilde_array)]
    vcoul = np.ascontiguousarray(prob.vcoul, dtype=np.float64)
    ach, asx = np.zeros(3, np.complex128), np.zeros(3, np.complex128)
    n1 = np.zeros(prob.number_bands, np.complex128) if want_n1 else None
    stat = np.zeros(1, np.complex128) if want_static else None
    fn = lib.sigma_gpp_halfsum_tensor if tensor else lib.sigma_gpp_halfsum_fp64
    st = fn(prob.number_bands, prob.nvband, prob.ncouls, prob.ngpown, prob.nstart,
            prob.nend, _ptr(inv), _ptr(indinv), _ptr(wx), prob.occ,
            *[_ptr(a) for a in arrs], _ptr(vcoul), _ptr(ach), _ptr(asx), _ptr(n1),
            _ptr(stat), stream)
    _check(st, fn.__name__)
    return ach, asx, n1, (stat[0] if want_static else None)


class GppHalfSumPlan:
    """Device-resident gppsum = 1 GPP (sigma_gpp_halfsum_plan_create / execute).
    flags: HALFSUM_STATIC (also achstemp), HALFSUM_GVEC_MAJOR (inputs in
    gppKerSeq.cpp's [ncouls][...] layout)."""

    def __init__(self, number_bands, nvband, ncouls, ngpown, inv_igp_index, indinv, flags=HALFSUM_STATIC):
        self.lib = load()
        self.inv = np.ascontiguousarray(inv_igp_index, dtype=np.int32)
        self.indinv = np.ascontiguousarray(indinv, dtype=np.int32)
        h = C.c_void_p()
        _check(self.lib.sigma_gpp_halfsum_plan_create(C.byref(h), number_bands, nvband, ncouls, ngpown, 0, 3,
                                                      _ptr(self.inv), _ptr(self.indinv), len(self.indinv),
                                                      flags), "sigma_gpp_halfsum_plan_create")
        self.handle = h

    def execute(self, wx, aqsm, aqsn, ieps, wt, vcoul, achtemp, asxtemp, acht_n1_loc=None, achstemp=None,
                occ=1.0, stream=0):
        _check(self.lib.sigma_gpp_halfsum_execute(
            self.handle, _dptr(wx), occ,
            *[_dptr(a) for a in (aqsm, aqsn, ieps, wt, vcoul, achtemp, asxtemp)],
            _dptr(acht_n1_loc), _dptr(achstemp), stream), "sigma_gpp_halfsum_execute")

    def close(self):
        if getattr(self, "handle", None):
            self.lib.sigma_gpp_halfsum_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GppRealPlan:
    """Device-resident real-valued GPP (sigma_gpp_real_plan_create / execute)."""

    def __init__(self, number_bands, nvband, ncouls, ngpown, inv_igp_index, indinv):
        self.lib = load()
        self.inv = np.ascontiguousarray(inv_igp_index, dtype=np.int32)
        self.indinv = np.ascontiguousarray(indinv, dtype=np.int32)
        h = C.c_void_p()
        _check(self.lib.sigma_gpp_real_plan_create(C.byref(h), number_bands, nvband, ncouls, ngpown, 0, 3,
                                                   _ptr(self.inv), _ptr(self.indinv), len(self.indinv)),
               "sigma_gpp_real_plan_create")
        self.handle = h

    def execute(self, wx, aqsm, aqsn, ieps, wt, vcoul, achtemp, asxtemp, acht_n1_loc=None, occ=1.0, stream=0):
        _check(self.lib.sigma_gpp_real_execute(self.handle, _dptr(wx), occ,
                                               *[_dptr(a) for a in (aqsm, aqsn, ieps, wt, vcoul, achtemp, asxtemp)],
                                               _dptr(acht_n1_loc), stream), "sigma_gpp_real_execute")

    def close(self):
        if getattr(self, "handle", None):
            self.lib.sigma_gpp_real_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GppPlan:
    """Device-resident GPP plan (sigma_gpp_plan_create / execute / destroy)."""

    def __init__(self, number_bands, nvband, ncouls, ngpown, inv_igp_index, indinv,
                 precision=PREC_FP64, nstart=0, nend=3):
        self.lib = load()
        self.inv = np.ascontiguousarray(inv_igp_index, dtype=np.int32)
        self.indinv = np.ascontiguousarray(indinv, dtype=np.int32)
        h = C.c_void_p()
        st = self.lib.sigma_gpp_plan_create(C.byref(h), number_bands, nvband, ncouls, ngpown, nstart,
                                            nend, _ptr(self.inv), _ptr(self.indinv), len(self.indinv),
                                            precision)
        _check(st, "sigma_gpp_plan_create")
        self.handle = h
        self.number_bands = number_bands

    def info(self):
        v = C.c_int()
        t = C.c_longlong()
        _check(self.lib.sigma_gpp_plan_info(self.handle, C.byref(v), C.byref(t)), "sigma_gpp_plan_info")
        return v.value, t.value

    def execute(self, wx, aqsm, aqsn, ieps, wt, vcoul, achtemp, asxtemp, acht_n1_loc=None,
                occ=1.0, wx_band_stride=0, stream=0):
        """All array arguments are device pointers (ints) or CUDA tensors."""
        st = self.lib.sigma_gpp_execute(self.handle, _ptr(wx) if not isinstance(wx, int) else wx,
                                        wx_band_stride, occ,
                                        *[a if isinstance(a, int) else _ptr(a)
                                          for a in (aqsm, aqsn, ieps, wt, vcoul, achtemp, asxtemp)],
                                        None if acht_n1_loc is None else
                                        (acht_n1_loc if isinstance(acht_n1_loc, int) else _ptr(acht_n1_loc)),
                                        stream)
        _check(st, "sigma_gpp_execute")

    def set_timing(self, enable=True):
        _check(self.lib.sigma_gpp_plan_set_timing(self.handle, int(enable)), "sigma_gpp_plan_set_timing")

    def timing(self):
        """dict(executions, main_ms, occupied_ms, other_ms, launches) summed
        over the executions recorded since timing was enabled / last read."""
        n = C.c_int()
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        l = C.c_int()
        _check(self.lib.sigma_gpp_plan_timing(self.handle, C.byref(n), C.byref(a), C.byref(b),
                                              C.byref(c), C.byref(l)), "sigma_gpp_plan_timing")
        return dict(executions=n.value, main_ms=a.value, occupied_ms=b.value, other_ms=c.value,
                    launches=l.value)

    def status(self, stream=0):
        """Device status of the last execution (0, or -5 after a bounded wait gave up)."""
        return self.lib.sigma_gpp_plan_status(self.handle, stream)

    def selftest_gate_timeout(self, wx, aqsm, aqsn, ieps, wt, vcoul, wait_polls, stream=0):
        """sigma_gpp_selftest_gate_timeout: the gated FP64 main pass with gate
        words nothing writes; returns the device status (-5 expected)."""
        return self.lib.sigma_gpp_selftest_gate_timeout(
            self.handle, *[a if isinstance(a, int) else _ptr(a) for a in (wx, aqsm, aqsn, ieps, wt, vcoul)],
            wait_polls, stream)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.sigma_gpp_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GppInstance(C.Structure):
    """sigma_gpp_instance: one GPP evaluation of a batch (device arrays, host index maps)."""
    _fields_ = [("number_bands", _I), ("nvband", _I), ("ncouls", _I), ("ngpown", _I),
                ("inv_igp_index", _P), ("indinv", _P), ("wx_array", _P), ("wx_band_stride", _I),
                ("occ", _D), ("aqsmtemp", _P), ("aqsntemp", _P), ("I_eps_array", _P),
                ("wtilde_array", _P), ("vcoul", _P), ("achtemp", _P), ("asxtemp", _P),
                ("acht_n1_loc", _P)]


def _dptr(a):
    return a if (a is None or isinstance(a, int)) else _ptr(a)


def _instance_array(instances, keep):
    arr = (GppInstance * len(instances))()
    for k, d in enumerate(instances):
        inv = np.ascontiguousarray(d["inv_igp_index"], dtype=np.int32)
        ind = np.ascontiguousarray(d["indinv"], dtype=np.int32)
        keep += [inv, ind]
        q = arr[k]
        q.number_bands, q.nvband, q.ncouls, q.ngpown = (d["number_bands"], d["nvband"],
                                                         d["ncouls"], d["ngpown"])
        q.inv_igp_index, q.indinv = _ptr(inv), _ptr(ind)
        q.wx_array = _dptr(d["wx_array"])
        q.wx_band_stride = d.get("wx_band_stride", 0)
        q.occ = d.get("occ", 1.0)
        for f in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul", "achtemp", "asxtemp"):
            setattr(q, f, _dptr(d[f]))
        q.acht_n1_loc = _dptr(d.get("acht_n1_loc"))
    return arr


def gpp_batched(instances, precision=PREC_FP64, stream=0):
    """One-shot sigma_gpp_batched: evaluates every instance and waits."""
    lib = load()
    keep = []
    arr = _instance_array(instances, keep)
    _check(lib.sigma_gpp_batched(len(instances), C.addressof(arr), precision, stream), "sigma_gpp_batched")


class GppBatch:
    """Many GPP instances through one work queue per pass
    (sigma_gpp_batch_create / execute / launch_graph / destroy).

    `instances` is a list of dicts with the sigma_gpp_instance fields: host
    index maps as numpy int arrays, every other array a CUDA tensor or a
    device pointer.  `tiles` (optional) gives the FP64 main-pass tile per
    instance (-1 library choice; per-band frequencies 0 = 32x32, 1 = 16x64,
    2 = 64x16; one frequency set 3 = 64x32, 4 = 32x64, 5 = 32x32, 6 =
    64x16).  `items_per_cta` / `tensor_split_tiles` (0: defaults) size the
    work items (sigma_gpp_batch_create_tuned)."""

    def __init__(self, instances, precision=PREC_FP64, tiles=None, items_per_cta=0, tensor_split_tiles=0):
        self.lib = load()
        self._keep = []
        arr = _instance_array(instances, self._keep)
        self._arr = arr
        t = None
        if tiles is not None:
            t = np.ascontiguousarray(tiles, dtype=np.int32)
            self._keep.append(t)
        h = C.c_void_p()
        st = self.lib.sigma_gpp_batch_create_tuned(C.byref(h), len(instances), C.addressof(arr), precision,
                                                   None if t is None else _ptr(t), int(items_per_cta),
                                                   int(tensor_split_tiles))
        _check(st, "sigma_gpp_batch_create_tuned")
        self.handle = h

    def info(self):
        """(terms, main-pass items, kernels per execution)."""
        t, i, l = C.c_longlong(), C.c_int(), C.c_int()
        _check(self.lib.sigma_gpp_batch_info(self.handle, C.byref(t), C.byref(i), C.byref(l)),
               "sigma_gpp_batch_info")
        return t.value, i.value, l.value

    def execute(self, stream=0):
        _check(self.lib.sigma_gpp_batch_execute(self.handle, stream), "sigma_gpp_batch_execute")

    def launch_graph(self, stream):
        _check(self.lib.sigma_gpp_batch_launch_graph(self.handle, stream), "sigma_gpp_batch_launch_graph")

    def status(self, stream=0):
        return self.lib.sigma_gpp_batch_status(self.handle, stream)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.sigma_gpp_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gpp_achstemp(prob, mode: int = FF_MODE_FP64, stream: int = 0):
    """Static remainder of the GPP sum (sigma_gpp_achstemp) on a
    workload.GppProblem: returns (achstemp, achstemp_n1[number_bands])."""
    lib = load()
    inv = np.ascontiguousarray(prob.inv_igp_index, dtype=np.int32)
    indinv = np.ascontiguousarray(prob.indinv, dtype=np.int32)
    arrs = [_c128(prob.aqsmtemp), _c128(prob.aqsntemp), _c128(prob.I_eps_array)]
    vcoul = np.ascontiguousarray(prob.vcoul, dtype=np.float64)
    out = np.zeros(1, np.complex128)
    n1 = np.zeros(prob.number_bands, np.complex128)
    st = lib.sigma_gpp_achstemp(prob.number_bands, prob.ncouls, prob.ngpown, _ptr(inv), _ptr(indinv),
                                *[_ptr(a) for a in arrs], _ptr(vcoul), _ptr(out), _ptr(n1), mode, stream)
    _check(st, "sigma_gpp_achstemp")
    return out[0], n1


class StaticPlan:
    """Device-resident static remainder (sigma_gpp_static_plan_create /
    sigma_gpp_static_execute; an FF plan underneath)."""

    def __init__(self, number_bands, ncouls, ngpown, inv_igp_index, indinv, mode=FF_MODE_FP64):
        self.lib = load()
        self.inv = np.ascontiguousarray(inv_igp_index, dtype=np.int32)
        self.indinv = np.ascontiguousarray(indinv, dtype=np.int32)
        h = C.c_void_p()
        _check(self.lib.sigma_gpp_static_plan_create(C.byref(h), number_bands, ncouls, ngpown,
                                                     _ptr(self.inv), _ptr(self.indinv), mode),
               "sigma_gpp_static_plan_create")
        self.handle = h

    def execute(self, aqsm, aqsn, ieps, vcoul, achstemp, achstemp_n1, stream=0):
        _check(self.lib.sigma_gpp_static_execute(self.handle, *[_dptr(a) for a in (aqsm, aqsn, ieps, vcoul,
                                                                                 achstemp, achstemp_n1)],
                                                 stream), "sigma_gpp_static_execute")

    def set_timing(self, enable=True):
        _check(self.lib.sigma_ff_plan_set_timing(self.handle, int(enable)), "sigma_ff_plan_set_timing")

    def timing(self):
        n, a, o, l = C.c_int(), C.c_double(), C.c_double(), C.c_int()
        _check(self.lib.sigma_ff_plan_timing(self.handle, C.byref(n), C.byref(a), C.byref(o), C.byref(l)),
               "sigma_ff_plan_timing")
        return dict(executions=n.value, main_ms=a.value, other_ms=o.value, launches=l.value)

    def status(self, stream=0):
        return self.lib.sigma_ff_plan_status(self.handle, stream)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.sigma_ff_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


FF_SIGMA_OUTPUTS = ("achsDtemp", "asxDtemp", "achDtemp", "achDtemp_cor", "achDtemp_corb", "ach2Dtemp")


def ff_sigma(prob, mode: int = FF_MODE_FP64, schdt="zero", stream: int = 0):
    """Full-frequency sigma (sigma_ff_sigma) on a workload.FFSigmaProblem.
    schdt: "zero" (the live Fortran's zeroed schDt_matrix), "compute" (the
    library contracts I_epsR itself), or a complex [number_bands][nfreq]
    array.  Returns a dict of the six outputs."""
    lib = load()
    p = prob
    c = lambda a: np.ascontiguousarray(a, dtype=np.complex128)
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    if isinstance(schdt, str):
        sd = np.zeros((p.number_bands, p.nfreq), np.complex128) if schdt == "zero" else None
    else:
        sd = c(schdt)
    args = [i32(p.inv_igp_index), i32(p.indinv), c(p.aqsmtemp), c(p.aqsntemp), c(p.I_epsR), c(p.I_epsA),
            f(p.vcoul), f(p.ekq), f(p.dFreqGrid), c(p.dFreqBrd), f(p.pref)]
    out = {k: np.zeros(1 if k == "achsDtemp" else p.nfreqeval, np.complex128) for k in FF_SIGMA_OUTPUTS}
    st = lib.sigma_ff_sigma(p.number_bands, p.nvband, p.ncouls, p.ngpown, p.nfreq, p.nfreqeval,
                            *[_ptr(a) for a in args], p.pref_zb, p.freqevalmin, p.freqevalstep, p.occ,
                            _ptr(sd), *[_ptr(out[k]) for k in FF_SIGMA_OUTPUTS], mode, stream)
    _check(st, "sigma_ff_sigma")
    out["achsDtemp"] = out["achsDtemp"][0]
    return out


class FfSigmaPlan:
    """Device-resident full-frequency sigma (sigma_ff_sigma_plan_create /
    sigma_ff_sigma_execute).  execute() takes device arrays (CUDA tensors or
    pointers) and a device output of 1 + 5 * nfreqeval complex values."""

    def __init__(self, number_bands, nvband, ncouls, ngpown, nfreq, nfreqeval, inv_igp_index, indinv,
                 mode=FF_MODE_FP64):
        self.lib = load()
        self.inv = np.ascontiguousarray(inv_igp_index, dtype=np.int32)
        self.indinv = np.ascontiguousarray(indinv, dtype=np.int32)
        self.nfreqeval = nfreqeval
        h = C.c_void_p()
        _check(self.lib.sigma_ff_sigma_plan_create(C.byref(h), number_bands, nvband, ncouls, ngpown, nfreq,
                                                   nfreqeval, _ptr(self.inv), _ptr(self.indinv), mode),
               "sigma_ff_sigma_plan_create")
        self.handle = h

    def execute(self, aqsm, aqsn, epsr, epsa, vcoul, ekq, grid, brd, pref, pref_zb, freqevalmin,
                freqevalstep, occ, schdt, out, stream=0):
        _check(self.lib.sigma_ff_sigma_execute(self.handle, *[_dptr(a) for a in (aqsm, aqsn, epsr, epsa, vcoul,
                                                                               ekq, grid, brd, pref)],
                                               pref_zb, freqevalmin, freqevalstep, occ, _dptr(schdt),
                                               _dptr(out), stream), "sigma_ff_sigma_execute")

    @staticmethod
    def unpack(out_host, nfreqeval):
        """Splits the output vector into the six named results."""
        z = np.asarray(out_host).view(np.complex128)
        res = {"achsDtemp": z[0]}
        for k, name in enumerate(FF_SIGMA_OUTPUTS[1:]):
            res[name] = z[1 + k * nfreqeval: 1 + (k + 1) * nfreqeval].copy()
        return res

    def set_timing(self, enable=True):
        _check(self.lib.sigma_ff_sigma_plan_set_timing(self.handle, int(enable)), "sigma_ff_sigma_plan_set_timing")

    def timing(self):
        n, a, o = C.c_int(), C.c_double(), C.c_double()
        _check(self.lib.sigma_ff_sigma_plan_timing(self.handle, C.byref(n), C.byref(a), C.byref(o)),
               "sigma_ff_sigma_plan_timing")
        return dict(contractions=n.value, contraction_ms=a.value, other_ms=o.value)

    def status(self, stream=0):
        return self.lib.sigma_ff_sigma_plan_status(self.handle, stream)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.sigma_ff_sigma_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ff_host(prob, mode: int = FF_MODE_FP64, stream: int = 0):
    """Host-pointer FF drop-in on a workload.FFProblem; returns schDt[nb][nfreq]."""
    lib = load()
    inv = np.ascontiguousarray(prob.inv_igp_index, dtype=np.int32)
    indinv = np.ascontiguousarray(prob.indinv, dtype=np.int32)
    epsr, aqsn, aqsm = _c128(prob.I_epsR), _c128(prob.aqsntemp), _c128(prob.aqsmtemp)
    out = np.zeros((prob.number_bands, prob.nfreq), np.complex128)
    st = lib.sigma_ff_schdt(prob.number_bands, prob.ncouls, prob.ngpown, prob.nfreq, _ptr(inv),
                            _ptr(indinv), _ptr(epsr), _ptr(aqsn), _ptr(aqsm), _ptr(out), mode, stream)
    _check(st, "sigma_ff_schdt")
    return out


class FfPlan:
    """Device-resident FF plan (sigma_ff_plan_create / execute / destroy)."""

    def __init__(self, number_bands, ncouls, ngpown, nfreq, inv_igp_index, indinv, mode=FF_MODE_FP64):
        self.lib = load()
        self.inv = np.ascontiguousarray(inv_igp_index, dtype=np.int32)
        self.indinv = np.ascontiguousarray(indinv, dtype=np.int32)
        h = C.c_void_p()
        _check(self.lib.sigma_ff_plan_create(C.byref(h), number_bands, ncouls, ngpown, nfreq,
                                             _ptr(self.inv), _ptr(self.indinv), mode),
               "sigma_ff_plan_create")
        self.handle = h

    def execute(self, epsr, aqsn, aqsm, schdt, stream=0):
        p = lambda a: a if isinstance(a, int) else _ptr(a)
        _check(self.lib.sigma_ff_execute(self.handle, p(epsr), p(aqsn), p(aqsm), p(schdt), stream),
               "sigma_ff_execute")

    def set_timing(self, enable=True):
        _check(self.lib.sigma_ff_plan_set_timing(self.handle, int(enable)), "sigma_ff_plan_set_timing")

    def timing(self):
        n, l = C.c_int(), C.c_int()
        a, b = C.c_double(), C.c_double()
        _check(self.lib.sigma_ff_plan_timing(self.handle, C.byref(n), C.byref(a), C.byref(b), C.byref(l)),
               "sigma_ff_plan_timing")
        return dict(executions=n.value, main_ms=a.value, other_ms=b.value, launches=l.value)

    def status(self, stream=0):
        return self.lib.sigma_ff_plan_status(self.handle, stream)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.sigma_ff_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fill_uniform(dst_ptr: int, count: int, dst_stride: int, seed: int, array_id: int,
                 draw_offset: int, draw_stride: int, lo: float, span: float, stream: int = 0):
    lib = load()
    _check(lib.sigma_fill_uniform(dst_ptr, count, dst_stride, seed, array_id, draw_offset,
                                  draw_stride, lo, span, stream), "sigma_fill_uniform")


def fill_complex_device(dst_ptr: int, n: int, seed: int, array_id: int, re: tuple, im: tuple,
                        stream: int = 0):
    """Device twin of workload.fill_complex."""
    fill_uniform(dst_ptr, n, 2, seed, array_id, 0, 2, float(re[0]), float(re[1]) - float(re[0]), stream)
    fill_uniform(dst_ptr + 8, n, 2, seed, array_id, 1, 2, float(im[0]), float(im[1]) - float(im[0]), stream)


def fill_real_device(dst_ptr: int, n: int, seed: int, array_id: int, lo: float, hi: float,
                     stream: int = 0):
    fill_uniform(dst_ptr, n, 1, seed, array_id, 0, 1, float(lo), float(hi) - float(lo), stream)


def fill_stress_device(wt_ptr: int, n: int, seed: int, array_id: int, wx, fraction=0.05,
                       width=1e-3, stream: int = 0):
    lib = load()
    w = np.ascontiguousarray(wx, dtype=np.float64)
    _check(lib.sigma_fill_stress(wt_ptr, n, seed, array_id, _ptr(w), len(w), fraction, width, stream),
           "sigma_fill_stress")


def measure_fma_peaks(stream: int = 0):
    """(fp64_tflops, fp32_tflops) measured on the current device."""
    lib = load()
    a = C.c_double()
    b = C.c_double()
    _check(lib.sigma_measure_fma_peaks(C.byref(a), C.byref(b), stream), "sigma_measure_fma_peaks")
    return a.value, b.value


def shutdown():
    if _lib is not None:
        _lib.sigma_shutdown()
