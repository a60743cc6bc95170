"""Host-side tests: the seeded generator, the C-ABI library's exports, and
argument validation that happens before any device work."""
import ctypes as C
import pathlib
import re

import numpy as np
import pytest

import workload as W

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_splitmix64_known_answer():
    # SplitMix64 from state 0 (Steele, Lea, Flood 2014): first output
    z = W._fmix(np.array([W.GOLDEN], dtype=np.uint64))
    assert int(z[0]) == 0xE220A8397B1DCDAF
    z2 = W._fmix(np.array([(2 * W.GOLDEN) & W.MASK], dtype=np.uint64))
    assert int(z2[0]) == 0x6E789E6AA1B965F4


def test_fill_is_deterministic_and_chunk_independent():
    a = W.fill_complex(5, W.AID_AQSM, 10_000, (-1, 1), (-1, 1))
    b = W.fill_complex(5, W.AID_AQSM, 10_000, (-1, 1), (-1, 1))
    assert np.array_equal(a, b)
    # a prefix equals a shorter fill (counter-based stream)
    c = W.fill_complex(5, W.AID_AQSM, 1234, (-1, 1), (-1, 1))
    assert np.array_equal(a[:1234], c)
    assert a.real.min() >= -1 and a.real.max() < 1
    w = W.fill_complex(1, W.AID_WTILDE, 50_000, (0.5, 5.0), (-0.1, 0.1))
    assert w.real.min() >= 0.5 and w.real.max() < 5 and np.abs(w.imag).max() <= 0.1
    # different array ids are different streams
    assert not np.array_equal(a, W.fill_complex(5, W.AID_AQSN, 10_000, (-1, 1), (-1, 1)))


def test_stress_moves_five_percent_near_poles():
    wt = W.fill_complex(2, W.AID_WTILDE, 200_000, (0.5, 5.0), (-0.1, 0.1))
    moved = W.stress_wtilde(wt, W.wx_frequencies(), 2)
    assert 0.045 < moved / wt.size < 0.055
    d = np.min(np.abs(wt.real[:, None] - W.wx_frequencies()[None, :]), axis=1)
    assert np.sum(d < 1e-3) >= moved


def test_reference_shapes_and_index_maps():
    sh = W.gpp_shape(**W.GPP_PRODUCTION)
    assert sh["ngpown"] == 1638
    inv, indinv = W.gpp_index_maps(32768, 1638)
    assert inv[0] == 32768 // 1638 and inv[-1] == 32768  # clamped to ncouls-1 downstream
    assert np.array_equal(W.wx_frequencies(), [3.0, 4.0, 5.0])
    shapes = W.batched_shapes()
    assert len(shapes) == 48
    for s in shapes:
        assert 64 <= s["number_bands"] <= 512 and 4096 <= s["ncouls"] <= 32768
        assert s["ncouls"] % 256 == 0 and 10 <= s["nodes_per_group"] <= 40 and 1 <= s["nvband"] <= 8


def _declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:int|const char\*|size_t|void)\s+(sigma_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    import build as B
    return B.build()


def test_library_exports_every_declared_symbol(libpath):
    lib = C.CDLL(str(libpath))
    declared = _declared_functions()
    assert len(declared) >= 10
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    import sigma_gb300
    assert set(declared) <= set(sigma_gb300.exported_symbols())


def _declared_arity():
    """Parameter count of every sigma_* prototype in include/*.h."""
    out = {}
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:int|const char\*|size_t|void)\s+(sigma_\w+)\s*\(([^;{]*?)\)\s*;",
                             text, flags=re.M | re.S):
            params = m.group(2).strip()
            out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_binding_argument_counts_match_headers():
    """Every ctypes binding takes exactly the parameters its C prototype declares."""
    import sigma_gb300
    arity = _declared_arity()
    bad = {n: (len(a), arity[n]) for n, (a, _) in sigma_gb300.SIGNATURES.items()
           if n in arity and len(a) != arity[n]}
    assert not bad, bad
    assert len(set(arity) & set(sigma_gb300.SIGNATURES)) >= 30


def test_status_strings(libpath):
    lib = C.CDLL(str(libpath))
    lib.sigma_status_string.restype = C.c_char_p
    assert lib.sigma_status_string(0) == b"ok"
    assert lib.sigma_status_string(-2) == b"index out of range"


def test_validation_precedes_device_work(libpath):
    """Bad shapes and out-of-bounds index maps are rejected on the host with
    the reference's failure points, before the device is touched."""
    lib = C.CDLL(str(libpath))
    f = lib.sigma_gpp_plan_create
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                  C.c_void_p, C.c_int, C.c_int]
    h = C.c_void_p()
    nc, ng = 64, 4
    inv = np.array([16, 32, 48, 64], np.int32)
    indinv = np.arange(nc, dtype=np.int32)
    args = lambda nb, nv, nc_, ng_, ns, ne, inv_, ind_, prec: f(C.byref(h), nb, nv, nc_, ng_, ns, ne,
                                                                inv_.ctypes.data, ind_.ctypes.data,
                                                                len(ind_), prec)
    assert args(2, 1, nc, ng, 0, 4, inv, indinv, 0) == -1      # nend - nstart != 3
    assert args(2, 3, nc, ng, 0, 3, inv, indinv, 0) == -1      # nvband > number_bands
    assert args(2, 1, 3, ng, 0, 3, inv, indinv, 0) == -1       # ngpown > ncouls
    assert args(2, 1, nc, ng, 0, 3, inv, indinv, 7) == -8      # unknown precision
    bad = inv.copy()
    bad[2] = 65                                                  # indigp > ncouls
    assert args(2, 1, nc, ng, 0, 3, bad, indinv, 0) == -2
    ind_bad = indinv.copy()
    ind_bad[32] = 64                                             # igp == ncouls
    assert args(2, 1, nc, ng, 0, 3, inv, ind_bad, 0) == -2
    st = args(2, 1, nc, ng, 0, 3, inv, indinv, 0)
    # valid arguments reach the device step: OK on a GPU host, no-device here
    assert st in (0, -7, -4)
    if st == 0:
        lib.sigma_gpp_plan_destroy.argtypes = [C.c_void_p]
        lib.sigma_gpp_plan_destroy(h)


def test_ff_validation_precedes_device_work(libpath):
    lib = C.CDLL(str(libpath))
    f = lib.sigma_ff_plan_create
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
    h = C.c_void_p()
    nc, ng = 64, 8
    inv = np.arange(ng, dtype=np.int32)
    indinv = np.arange(nc, dtype=np.int32)
    call = lambda nb, nc_, ng_, nf, inv_, ind_, mode: f(C.byref(h), nb, nc_, ng_, nf, inv_.ctypes.data,
                                                       ind_.ctypes.data, mode)
    assert call(4, nc, 65, 2, np.arange(65, dtype=np.int32), indinv, 0) == -1  # ngpown > ncouls
    assert call(4, nc, ng, 0, inv, indinv, 0) == -1                             # no frequency
    assert call(4, nc, ng, 2, inv, indinv, 5) == -8                             # unknown mode
    bad = inv.copy()
    bad[1] = nc                                  # indinv read past its end
    assert call(4, nc, ng, 2, bad, indinv, 0) == -2
    ind_bad = indinv.copy()
    ind_bad[3] = -1                              # igp outside [0, ncouls)
    assert call(4, nc, ng, 2, inv, ind_bad, 1) == -2
    st = call(4, nc, ng, 2, inv, indinv, 0)
    assert st in (0, -7, -4)
    if st == 0:
        lib.sigma_ff_plan_destroy.argtypes = [C.c_void_p]
        lib.sigma_ff_plan_destroy(h)


def test_batch_validation_precedes_device_work(libpath):
    """sigma_gpp_batch_create checks every instance on the host first."""
    import sigma_gb300 as S
    lib = C.CDLL(str(libpath))
    f = lib.sigma_gpp_batch_create
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    nc, ng = 64, 4
    inv, indinv = W.gpp_index_maps(nc, ng)
    fake = 256  # device pointers are not touched before the device step
    good = dict(number_bands=2, nvband=1, ncouls=nc, ngpown=ng, inv_igp_index=inv, indinv=indinv,
                wx_array=fake, aqsmtemp=fake, aqsntemp=fake, I_eps_array=fake, wtilde_array=fake,
                vcoul=fake, achtemp=fake, asxtemp=fake)
    h = C.c_void_p()

    def create(insts, prec=0, tiles=None):
        keep = []
        arr = S._instance_array(insts, keep)
        t = None if tiles is None else np.asarray(tiles, np.int32)
        return f(C.byref(h), len(insts), C.addressof(arr), prec, None if t is None else t.ctypes.data)

    assert create([]) == -1
    assert create([good, dict(good, ngpown=65, inv_igp_index=np.arange(65, dtype=np.int32))]) == -1
    assert create([good, dict(good, inv_igp_index=np.array([16, 32, 65, 64], np.int32))]) == -2
    assert create([good, dict(good, aqsntemp=None)]) == -6
    assert create([good], prec=3) == -8
    assert create([good, dict(good, wx_band_stride=3)], prec=2) == -8   # tensor needs shared frequencies
    assert create([good, good], tiles=[0, 5]) == -8
    assert create([dict(good, wx_band_stride=2)]) == -1
    assert create([good, good], tiles=[1, -1]) == -8   # per-band-kernel tile, shared frequencies
    assert create([good, dict(good, wx_band_stride=3)], tiles=[4, 0]) == -8  # mixed families
    # the tuned entry: negative sizing is an invalid shape, checked first
    g = lib.sigma_gpp_batch_create_tuned
    g.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int]
    keep = []
    arr = S._instance_array([good], keep)
    assert g(C.byref(h), 1, C.addressof(arr), 0, None, -1, 0) == -1
    assert g(C.byref(h), 1, C.addressof(arr), 2, None, 0, -3) == -1
    st = create([good, good], tiles=[4, -1])
    assert st in (0, -7, -4)
    if st == 0:
        lib.sigma_gpp_batch_destroy.argtypes = [C.c_void_p]
        lib.sigma_gpp_batch_destroy(h)


def test_tile_table_covers_every_shape_class():
    import autotune as A
    t = A.load_table()
    assert t is not None and t["device"].startswith("NVIDIA")
    keys = {A.shape_class(nb, ng) for nb in range(1, 200) for ng in range(1, 200)}
    assert len(keys) == 16
    for family, key in A.TABLE_KEY.items():
        if key not in t:
            continue
        assert keys == set(t[key])
        assert all(v in A.FAMILIES[family] for v in t[key].values())
        timings = t["timings" if family == "shared" else "timings_per_band"]
        # the tuned tile of a class is the fastest one it timed
        for k, v in t[key].items():
            ms = timings[k]["ms"]
            assert A.TILES[v] == min(ms, key=ms.get)
    assert A.shape_class(16, 16) == "b0c0" and A.shape_class(17, 64) == "b1c3"
    for s in W.batched_shapes():
        assert A.tile_for(s["number_bands"], s["ngpown"]) in (-1, 3, 4, 5, 6)
        assert A.tile_for(s["number_bands"], s["ngpown"], shared=False) in (-1, 0, 1, 2)
    # every form's work sizing: a tuned candidate, the fastest accepted one
    for form, key in A.SIZING_KEY.items():
        v = A.sizing_for(form, t)
        if key not in t:
            assert v == 0
            continue
        assert v in A.SIZING_CANDIDATES[form]
        ms = {int(k): m for k, m in t["sizing_timings_ms"][form].items() if m is not None}
        assert v == min(ms, key=ms.get)
