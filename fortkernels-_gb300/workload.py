"""Sigma workloads: the mini-app's constant fill and seeded synthetic fills.

The reference has no dataset; its drivers fill every array with constants
(BGW-Kernels/gppKer.cpp:275-299, FFKer_cori/ffKernel.cpp:398-433) and its job
scripts name the production shape `512 2 32768 20` (run_gppKerHSW.slurm:67).
The seeded fills here stand in for real BerkeleyGW matrices with the shapes
and value ranges of those runs.

Random numbers come from SplitMix64 (Steele, Lea and Flood, "Fast splittable
pseudorandom number generators", OOPSLA 2014) used as a counter-based stream:
draw i of stream (seed, array_id) is the SplitMix64 finaliser applied to
``s0 + (i + 1) * 0x9E3779B97F4A7C15`` with ``s0 = fmix(seed * K + array_id)``.
A draw becomes a double in [0, 1) as ``(draw >> 11) * 2**-53`` and a value in
[lo, hi) as ``lo + (hi - lo) * u`` with two separate roundings.  Complex
element k takes its real part from draw 2k and its imaginary part from draw
2k+1.  The device fill kernel (csrc/fill.cu) computes the same bits.
"""
from __future__ import annotations

import dataclasses
import numpy as np

GOLDEN = 0x9E3779B97F4A7C15
SEED_K = 0xD1342543DE82EF95
M1 = 0xBF58476D1CE4E5B9
M2 = 0x94D049BB133111EB
MASK = (1 << 64) - 1

# array ids of the seeded streams
AID_AQSM, AID_AQSN, AID_IEPS, AID_WTILDE, AID_VCOUL = 1, 2, 3, 4, 5
AID_STRESS, AID_IEPSR, AID_IEPSA, AID_SHAPES = 6, 7, 8, 100

# physics constants of the mini-app (BGW-Kernels/gppKer.cpp:178-201)
E_LK, DW, E_N1KQ, TO1 = 10.0, 1.0, 6.0, 1e-6
LIMITONE = 1.0 / (TO1 * 4.0)
LIMITTWO = 0.5 ** 2

_CHUNK = 1 << 22


def _fmix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * np.uint64(M1)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(M2)
    return z ^ (z >> np.uint64(31))


def stream_state(seed: int, array_id: int) -> int:
    """Initial SplitMix64 state of stream (seed, array_id)."""
    z = np.array([(seed * SEED_K + array_id) & MASK], dtype=np.uint64)
    return int(_fmix(z)[0])


def draws_u01(seed: int, array_id: int, start: int, count: int) -> np.ndarray:
    """Uniform doubles in [0, 1) for draws start..start+count-1 of a stream."""
    s0 = np.uint64(stream_state(seed, array_id))
    i = np.arange(start + 1, start + count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = _fmix(s0 + i * np.uint64(GOLDEN))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def fill_real(seed: int, array_id: int, n: int, lo: float, hi: float, start: int = 0) -> np.ndarray:
    """float64 elements start..start+n-1 of a real array (draw k -> element k)."""
    out = np.empty(n, dtype=np.float64)
    span = float(hi) - float(lo)
    for s in range(0, n, _CHUNK):
        c = min(_CHUNK, n - s)
        out[s:s + c] = lo + span * draws_u01(seed, array_id, start + s, c)
    return out


def fill_complex(seed: int, array_id: int, n: int, re: tuple, im: tuple, start: int = 0) -> np.ndarray:
    """complex128 elements start..start+n-1: real part from even draws,
    imaginary part from odd draws."""
    out = np.empty(n, dtype=np.complex128)
    view = out.view(np.float64)
    rspan = float(re[1]) - float(re[0])
    ispan = float(im[1]) - float(im[0])
    for s in range(0, n, _CHUNK // 2):
        c = min(_CHUNK // 2, n - s)
        u = draws_u01(seed, array_id, 2 * (start + s), 2 * c)
        view[2 * s:2 * (s + c):2] = re[0] + rspan * u[0::2]
        view[2 * s + 1:2 * (s + c):2] = im[0] + ispan * u[1::2]
    return out


def wx_frequencies(nend: int = 3, nstart: int = 0) -> np.ndarray:
    """wx_array of BGW-Kernels/gppKer.cpp:310-314 (e_lk - e_n1kq + dw*((iw+1)-2), |wx| >= to1)."""
    wx = np.array([E_LK - E_N1KQ + DW * ((iw + 1) - 2) for iw in range(nstart, nend)], dtype=np.float64)
    wx[np.abs(wx) < TO1] = TO1
    return wx


def gpp_index_maps(ncouls: int, ngpown: int):
    """inv_igp_index / indinv of BGW-Kernels/gppKer.cpp:294-299."""
    inv = ((np.arange(ngpown, dtype=np.int64) + 1) * ncouls // ngpown).astype(np.int32)
    indinv = np.arange(ncouls, dtype=np.int32)
    return inv, indinv


@dataclasses.dataclass
class GppProblem:
    number_bands: int
    nvband: int
    ncouls: int
    ngpown: int
    inv_igp_index: np.ndarray
    indinv: np.ndarray
    wx_array: np.ndarray
    aqsmtemp: np.ndarray       # complex128 [NB][NC]
    aqsntemp: np.ndarray       # complex128 [NB][NC]
    I_eps_array: np.ndarray    # complex128 [NG][NC]
    wtilde_array: np.ndarray   # complex128 [NG][NC]
    vcoul: np.ndarray          # float64 [NC]
    occ: float = 1.0
    nstart: int = 0
    nend: int = 3

    @property
    def terms(self) -> int:
        return self.number_bands * self.ngpown * self.ncouls * (self.nend - self.nstart)


def gpp_shape(number_bands, nvband, ncouls, nodes_per_group):
    """ngpown as the reference derives it (BGW-Kernels/gppKer.cpp:175-176, npes = 1)."""
    return dict(number_bands=number_bands, nvband=nvband, ncouls=ncouls,
                ngpown=ncouls // nodes_per_group)


def gpp_constant(number_bands, nvband, ncouls, nodes_per_group) -> GppProblem:
    """The mini-app's own fill: every complex is 0.5+0.5i, vcoul = 1."""
    sh = gpp_shape(number_bands, nvband, ncouls, nodes_per_group)
    nb, nc, ng = sh["number_bands"], ncouls, sh["ngpown"]
    inv, indinv = gpp_index_maps(nc, ng)
    a = np.full((nb, nc), 0.5 + 0.5j)
    e = np.full((ng, nc), 0.5 + 0.5j)
    return GppProblem(nb, nvband, nc, ng, inv, indinv, wx_frequencies(),
                      a, a.copy(), e, e.copy(), np.ones(nc))


def stress_wtilde(wtilde: np.ndarray, wx: np.ndarray, seed: int, fraction: float = 0.05,
                  width: float = 1e-3) -> int:
    """Moves `fraction` of the wtilde elements to re = wx_k +- U(0, width) in place.

    Element k uses draws 3k, 3k+1, 3k+2 of stream (seed, AID_STRESS): selected
    when the first is below `fraction`; the second picks k uniformly among the
    frequencies, the third the signed offset.  Returns the count moved."""
    flat = wtilde.reshape(-1)
    view = flat.view(np.float64)
    moved = 0
    n = flat.size
    step = _CHUNK // 4
    nw = len(wx)
    for s in range(0, n, step):
        c = min(step, n - s)
        u = draws_u01(seed, AID_STRESS, 3 * s, 3 * c).reshape(c, 3)
        sel = np.nonzero(u[:, 0] < fraction)[0]
        k = np.minimum((u[sel, 1] * nw).astype(np.int64), nw - 1)
        off = (2.0 * u[sel, 2] - 1.0) * width
        view[2 * (s + sel)] = wx[k] + off
        moved += sel.size
    return moved


def gpp_random(number_bands, nvband, ncouls, ngpown, seed, stress=False,
               nodes_per_group=None) -> GppProblem:
    """Seeded fill with the production value ranges: aqsm, aqsn, I_eps ~ U(-1,1)
    per part, wtilde re ~ U(0.5,5) and im ~ U(-0.1,0.1), vcoul ~ U(0.1,10);
    index maps and frequencies as the mini-app builds them."""
    if nodes_per_group is not None:
        ngpown = ncouls // nodes_per_group
    nb, nc, ng = number_bands, ncouls, ngpown
    inv, indinv = gpp_index_maps(nc, ng)
    wx = wx_frequencies()
    aqsm = fill_complex(seed, AID_AQSM, nb * nc, (-1, 1), (-1, 1)).reshape(nb, nc)
    aqsn = fill_complex(seed, AID_AQSN, nb * nc, (-1, 1), (-1, 1)).reshape(nb, nc)
    ieps = fill_complex(seed, AID_IEPS, ng * nc, (-1, 1), (-1, 1)).reshape(ng, nc)
    wt = fill_complex(seed, AID_WTILDE, ng * nc, (0.5, 5.0), (-0.1, 0.1)).reshape(ng, nc)
    if stress:
        stress_wtilde(wt, wx, seed)
    vcoul = fill_real(seed, AID_VCOUL, nc, 0.1, 10.0)
    return GppProblem(nb, nvband, nc, ng, inv, indinv, wx, aqsm, aqsn, ieps, wt, vcoul)


# ---------------------------------------------------------------- named configs
GPP_SMALL = dict(number_bands=128, nvband=2, ncouls=8192, nodes_per_group=20)        # constant fill
GPP_PRODUCTION = dict(number_bands=512, nvband=2, ncouls=32768, nodes_per_group=20)  # seed 1
GPP_STRESS_SEED = 2
GPP_PRODUCTION_SEED = 1


def batched_shapes(n_instances=48, seed=3):
    """Uneven instance shapes: NB ~ U{64..512}, NC ~ U{4096..32768} rounded to
    256, nodes_per_group ~ U{10..40}, nvband ~ U{1..8}; instance i is filled
    with seed 1000 + i."""
    u = draws_u01(seed, AID_SHAPES, 0, 4 * n_instances).reshape(n_instances, 4)
    out = []
    for i in range(n_instances):
        nb = 64 + int(u[i, 0] * (512 - 64 + 1))
        nc = 4096 + int(u[i, 1] * (32768 - 4096 + 1))
        nc = max(256, min(32768, int(round(nc / 256.0)) * 256))
        npg = 10 + int(u[i, 2] * (40 - 10 + 1))
        nvb = 1 + int(u[i, 3] * 8)
        out.append(dict(number_bands=nb, nvband=nvb, ncouls=nc, ngpown=nc // npg,
                        nodes_per_group=npg, seed=1000 + i))
    return out


@dataclasses.dataclass
class FFProblem:
    number_bands: int
    ncouls: int
    ngpown: int
    nfreq: int
    inv_igp_index: np.ndarray
    indinv: np.ndarray
    I_epsR: np.ndarray     # complex128 [nfreq][NG][NC]
    aqsntemp: np.ndarray   # complex128 [NB][NC]
    aqsmtemp: np.ndarray   # complex128 [NB][NC]

    @property
    def flops(self) -> int:
        return 8 * self.nfreq * self.ngpown * self.number_bands * self.ncouls


FF_PRODUCTION = dict(number_bands=512, ncouls=16384, ngpown=820, nfreq=15)
FF_SEED = 4


def ff_index_maps(ncouls, ngpown):
    """inv_igp_index[i] = i, indinv[i] = i (FFKer_cori/ffKernel.cpp:403-407)."""
    return np.arange(ngpown, dtype=np.int32), np.arange(ncouls, dtype=np.int32)


def ff_constant(number_bands, ncouls, ngpown, nfreq) -> FFProblem:
    inv, indinv = ff_index_maps(ncouls, ngpown)
    a = np.full((number_bands, ncouls), 0.5 + 0.5j)
    r = np.full((nfreq, ngpown, ncouls), 0.5 + 0.5j)
    return FFProblem(number_bands, ncouls, ngpown, nfreq, inv, indinv, r, a, a.copy())


def ff_random(number_bands, ncouls, ngpown, nfreq, seed) -> FFProblem:
    inv, indinv = ff_index_maps(ncouls, ngpown)
    nb, nc = number_bands, ncouls
    aqsm = fill_complex(seed, AID_AQSM, nb * nc, (-1, 1), (-1, 1)).reshape(nb, nc)
    aqsn = fill_complex(seed, AID_AQSN, nb * nc, (-1, 1), (-1, 1)).reshape(nb, nc)
    r = fill_complex(seed, AID_IEPSR, nfreq * ngpown * nc, (-1, 1), (-1, 1)).reshape(nfreq, ngpown, nc)
    return FFProblem(nb, nc, ngpown, nfreq, inv, indinv, r, aqsn, aqsm)


# ---------------------------------------------------------------- FF sigma
@dataclasses.dataclass
class FFSigmaProblem:
    """Inputs of the full-frequency sigma band loop (ffkernel.deslippe.best.f90
    :201-626) in the C layouts of FFKer_cori/ffKernel.cpp."""
    number_bands: int
    nvband: int
    ncouls: int
    ngpown: int
    nfreq: int
    nfreqeval: int
    inv_igp_index: np.ndarray
    indinv: np.ndarray
    aqsmtemp: np.ndarray    # complex128 [NB][NC]
    aqsntemp: np.ndarray    # complex128 [NB][NC]
    I_epsR: np.ndarray      # complex128 [nfreq][NG][NC]
    I_epsA: np.ndarray      # complex128 [nfreq][NG][NC]
    vcoul: np.ndarray       # float64 [NC]
    ekq: np.ndarray         # float64 [NB]
    dFreqGrid: np.ndarray   # float64 [nfreq]
    dFreqBrd: np.ndarray    # complex128 [nfreq]
    pref: np.ndarray        # float64 [nfreq]
    pref_zb: float = 0.5 / 3.14
    freqevalmin: float = 0.0
    freqevalstep: float = 0.5
    occ: float = 1.0

    def ff_problem(self) -> "FFProblem":
        """The schDt contraction of the same inputs (I_epsR)."""
        return FFProblem(self.number_bands, self.ncouls, self.ngpown, self.nfreq, self.inv_igp_index,
                         self.indinv, self.I_epsR, self.aqsntemp, self.aqsmtemp)


def ff_sigma_grid(number_bands, nfreq):
    """The mini-app's energies and frequency grid (ffkernel.deslippe.best.f90
    :103-150): ekq[n1] = -10 + n1, dFreqGrid[f] = 2 f, pref[f] = (grid[f+1] -
    grid[f]) / 3.14 with both ends halved, dFreqBrd = 0.1 i."""
    ekq = -10.0 + np.arange(number_bands, dtype=np.float64)
    grid = 2.0 * np.arange(nfreq, dtype=np.float64)
    pref = np.empty(nfreq)
    pref[:-1] = (grid[1:] - grid[:-1]) / 3.14
    pref[-1] = pref[-2]
    pref[0] *= 0.5
    pref[-1] *= 0.5
    brd = np.full(nfreq, 0.1j)
    return ekq, grid, brd, pref


def ff_sigma_constant(number_bands, nvband, ncouls, ngpown, nfreq, nfreqeval) -> FFSigmaProblem:
    """The mini-app's own fill: aqsm = aqsn = I_epsR = 0.5+0.5i, I_epsA =
    0.5-0.5i, vcoul = 1, identity index maps."""
    inv, indinv = ff_index_maps(ncouls, ngpown)
    ekq, grid, brd, pref = ff_sigma_grid(number_bands, nfreq)
    a = np.full((number_bands, ncouls), 0.5 + 0.5j)
    r = np.full((nfreq, ngpown, ncouls), 0.5 + 0.5j)
    return FFSigmaProblem(number_bands, nvband, ncouls, ngpown, nfreq, nfreqeval, inv, indinv, a,
                          a.copy(), r, np.conj(r), np.ones(ncouls), ekq, grid, brd, pref)


def ff_sigma_random(number_bands, nvband, ncouls, ngpown, nfreq, nfreqeval, seed) -> FFSigmaProblem:
    """Seeded inputs: aqsm, aqsn, I_epsR, I_epsA ~ U(-1,1) per part, vcoul ~
    U(0.1,10); energies and grid as the mini-app sets them."""
    inv, indinv = ff_index_maps(ncouls, ngpown)
    nb, nc = number_bands, ncouls
    ekq, grid, brd, pref = ff_sigma_grid(nb, nfreq)
    aqsm = fill_complex(seed, AID_AQSM, nb * nc, (-1, 1), (-1, 1)).reshape(nb, nc)
    aqsn = fill_complex(seed, AID_AQSN, nb * nc, (-1, 1), (-1, 1)).reshape(nb, nc)
    r = fill_complex(seed, AID_IEPSR, nfreq * ngpown * nc, (-1, 1), (-1, 1)).reshape(nfreq, ngpown, nc)
    a = fill_complex(seed, AID_IEPSA, nfreq * ngpown * nc, (-1, 1), (-1, 1)).reshape(nfreq, ngpown, nc)
    vcoul = fill_real(seed, AID_VCOUL, nc, 0.1, 10.0)
    return FFSigmaProblem(nb, nvband, nc, ngpown, nfreq, nfreqeval, inv, indinv, aqsm, aqsn, r, a, vcoul,
                          ekq, grid, brd, pref)


# ---------------------------------------------------------------- real-valued GPP
def gpp_real_constant(number_bands, nvband, ncouls, nodes_per_group) -> GppProblem:
    """gppKer_real.cpp's own fill (:262-282): every array 0.5, vcoul 1, the
    mini-app's index maps and frequencies.  Arrays are float64."""
    sh = gpp_shape(number_bands, nvband, ncouls, nodes_per_group)
    nb, nc, ng = number_bands, ncouls, sh["ngpown"]
    inv, indinv = gpp_index_maps(nc, ng)
    a = np.full((nb, nc), 0.5)
    e = np.full((ng, nc), 0.5)
    return GppProblem(nb, nvband, nc, ng, inv, indinv, wx_frequencies(), a, a.copy(), e, e.copy(),
                      np.ones(nc))


def gpp_real_random(number_bands, nvband, ncouls, ngpown, seed) -> GppProblem:
    """Seeded real inputs: aqsm, aqsn, I_eps ~ U(-1,1), wtilde ~ U(0.5,5),
    vcoul ~ U(0.1,10); index maps and frequencies of the mini-app."""
    nb, nc, ng = number_bands, ncouls, ngpown
    inv, indinv = gpp_index_maps(nc, ng)
    aqsm = fill_real(seed, AID_AQSM, nb * nc, -1, 1).reshape(nb, nc)
    aqsn = fill_real(seed, AID_AQSN, nb * nc, -1, 1).reshape(nb, nc)
    ieps = fill_real(seed, AID_IEPS, ng * nc, -1, 1).reshape(ng, nc)
    wt = fill_real(seed, AID_WTILDE, ng * nc, 0.5, 5.0).reshape(ng, nc)
    vcoul = fill_real(seed, AID_VCOUL, nc, 0.1, 10.0)
    return GppProblem(nb, nvband, nc, ng, inv, indinv, wx_frequencies(), aqsm, aqsn, ieps, wt, vcoul)
