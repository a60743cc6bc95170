// CPU oracle of the gppsum = 1 ("half sum") GPP variant.  TEST
// INFRASTRUCTURE ONLY: tests/ and bench.py's CPU-baseline leg load it; the
// product library never links or calls it.
//
// The one statement of gppsum = 1 in the reference that builds on its own
// is gppKerSeq.cpp (the Kokkos forms need Kokkos).  This file restates it
// per term with std::complex<double> in that file's operation order, in the
// library's band-major layout (aqsm[n1][ig], I_eps[my_igp][ig]; the
// reference stores the transposes, aqsmtemp[ig][n1] and
// I_eps_array[ig][my_igp]), and sums in a fixed order with double-double
// accumulators.
//
//   occupied bands     flagOCC_solver, gppsum branch     gppKerSeq.cpp:76-139
//   other bands        noflagOCC_solver, gppsum branch   gppKerSeq.cpp:193-242
//                      driven in 512-wide blocks         gppKerSeq.cpp:457-470
//   static remainder   reduce_achstemp, gppsum branch    gppKerSeq.cpp:13-72
//   epilogue           gppKerSeq.cpp:473-488
//   index mapping      gppKerSeq.cpp:425-431 (as gppKer.cpp:322-328)
//
// Build with -ffp-contract=off (oracle/build.py).

#include <complex>
#include <cmath>
#include <cstdint>
#include <vector>
#include <omp.h>

namespace {

using cd = std::complex<double>;

constexpr double kTo1 = 1e-6;
constexpr double kGamma = 0.5;
constexpr double kLimitOne = 1.0 / (kTo1 * 4.0);
constexpr double kLimitTwo = 0.5 * 0.5;
constexpr int kIgBlk = 512;

struct DD {
  double hi = 0.0, lo = 0.0;
};
inline void dd_add(DD& x, double y) {
  const double s = x.hi + y;
  const double bv = s - x.hi;
  double e = (x.hi - (s - bv)) + (y - bv);
  e += x.lo;
  x.hi = s + e;
  x.lo = e - (x.hi - s);
}
struct CDD {
  DD re, im;
  void add(const cd& v) {
    dd_add(re, v.real());
    dd_add(im, v.imag());
  }
  void add(const CDD& v) {
    dd_add(re, v.re.hi);
    dd_add(re, v.re.lo);
    dd_add(im, v.im.hi);
    dd_add(im, v.im.lo);
  }
  cd value() const { return cd(re.hi + re.lo, im.hi + im.lo); }
};

// igp of column my_igp: -1 skipped, -2 an index the reference would read out
// of bounds (the library reports it as an error).
inline int map_igp(const int* inv, const int* indinv, int indinv_len, int nc, int my_igp) {
  const int indigp = inv[my_igp];
  if (indigp < 0 || indigp > nc) return -2;
  int igp;
  if (indigp == nc) {
    igp = nc - 1;
  } else {
    if (indigp >= indinv_len) return -2;
    igp = indinv[indigp];
  }
  if (igp > nc || igp < 0) return -1;
  if (igp == nc) return -2;
  return igp;
}

// One g-vector of the non-occupied half sum (gppKerSeq.cpp:210-223):
// sch = delw I_eps when the (inverted) test passes, delw = wtilde / wdiff.
inline cd half_sch(double wxt, const cd& wtilde, const cd& ieps) {
  const cd wdiff = wxt - wtilde;
  const cd delw = wtilde / wdiff;
  const double delw2 = std::real(delw * std::conj(delw));
  const double wdiffr = std::real(wdiff * std::conj(wdiff));
  const double mult = (std::abs(wdiffr) < kLimitTwo || delw2 > kLimitOne) ? 1.0 : 0.0;
  return delw * ieps * mult;
}

// scht of one (n1, my_igp, iw) block call of noflagOCC_solver with gppsum = 1
// (gppKerSeq.cpp:206-242): g-vectors [igbeg, min(igend, igmax - 1)), plus
// g-vector igmax alone when igend == igmax - 1.
inline void half_block(int igbeg, int igend, int igmax, double wxt, const cd* wrow,
                       const cd* erow, const cd* nrow, const cd* mrow, const cd& mygpvar1,
                       const cd& mygpvar2, CDD& acc) {
  const int stop = std::min(igend, igmax - 1);
  for (int ig = igbeg; ig < stop; ++ig) {
    const cd matngmatmgp = nrow[ig] * mygpvar1;
    const cd sch = half_sch(wxt, wrow[ig], erow[ig]);
    acc.add(matngmatmgp * sch + std::conj(mrow[ig]) * mygpvar2 * std::conj(sch));
  }
  if (igend == igmax - 1) {
    const int ig = igmax;
    const cd matngmatmgp = nrow[ig] * mygpvar1;
    const cd sch = half_sch(wxt, wrow[ig], erow[ig]);
    acc.add(matngmatmgp * sch);
  }
}

// ssxt and scht of one (n1, my_igp, iw) for an occupied band
// (flagOCC_solver with gppsum = 1, gppKerSeq.cpp:88-139).
inline void half_occ(double wxt, int igmax, int igp, const cd* wrow, const cd* erow,
                     const cd* nrow, const cd* mrow, const cd& mygpvar1, const cd& mygpvar2,
                     CDD& ssxt, CDD& scht) {
  cd matngpmatmg(0.0, 0.0);
  for (int ig = 0; ig < igmax; ++ig) {
    const cd wtilde = wrow[ig];
    const cd wtilde2 = wtilde * wtilde;  // std::pow(w, 2) in libstdc++ is 1 * (w * w)
    const cd omega2 = wtilde2 * erow[ig];
    if (std::abs(omega2) < kTo1) break;
    const cd matngmatmgp = nrow[ig] * mygpvar1;
    if (ig != igp) matngpmatmg = std::conj(mrow[ig]) * mygpvar2;
    const cd halfinvwtilde = 0.5 / wtilde;
    const cd delw = (wxt - wtilde) * halfinvwtilde;
    const double adelw = std::abs(delw);
    const double delw2 = adelw * adelw;
    cd sch, ssx;
    if ((std::abs(wxt - wtilde) < kGamma) || (delw2 < kTo1)) {
      sch = cd(0.0, 0.0);
      ssx = std::abs(wtilde) > kTo1 ? -omega2 / (4.0 * wtilde2 * (1.0 + delw)) : cd(0.0, 0.0);
    } else {
      sch = wtilde * erow[ig] / (wxt - wtilde);
      ssx = omega2 / (wxt * wxt - wtilde2);
    }
    // the ssxcutoff test of :120-121 compares abs(wxt) < 0 and never fires
    if (ig != igp - 1) {
      ssxt.add(matngmatmgp * ssx + matngpmatmg * std::conj(ssx));
      scht.add(matngmatmgp * sch + matngpmatmg * std::conj(sch));
    } else {
      ssxt.add(matngmatmgp * ssx);
      scht.add(matngmatmgp * sch);
    }
  }
}

}  // namespace

extern "C" {

// gppsum = 1 GPP sum of gppKerSeq.cpp in band-major layout: complex128
// aqsm/aqsn [nb][nc], I_eps/wtilde [ng][nc], vcoul [nc], wx [3].  Outputs
// achtemp[3], asxtemp[3]; acht_n1_loc[nb], achstemp[1] (the static remainder
// summed over every band and column, gppKerSeq.cpp:412 accumulates it over
// the band loop), col_sch/col_ssx [nb][ng][3] (sch_array and ssx_array of
// every (n1, my_igp), before vcoul) are optional.  Only bands [band_begin,
// band_end) are summed (acht_n1_loc and the column arrays are written for
// those bands).  Returns 0 or a negative error code.
int oracle_gpp_halfsum(int number_bands, int nvband, int ncouls, int ngpown,
                       const int* inv_igp_index, const int* indinv, int indinv_len,
                       const double* wx, double occ, const double* aqsmtemp,
                       const double* aqsntemp, const double* I_eps_array,
                       const double* wtilde_array, const double* vcoul, double* achtemp,
                       double* asxtemp, double* acht_n1_loc, double* achstemp, double* col_sch,
                       double* col_ssx, int nthreads, int band_begin, int band_end) {
  if (!inv_igp_index || !indinv || !wx || !aqsmtemp || !aqsntemp || !I_eps_array ||
      !wtilde_array || !vcoul || !achtemp || !asxtemp)
    return -6;
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0 || nvband < 0 || nvband > number_bands ||
      band_begin < 0 || band_end > number_bands || band_begin > band_end)
    return -1;
  std::vector<int> igp_of(ngpown);
  for (int g = 0; g < ngpown; ++g) {
    igp_of[g] = map_igp(inv_igp_index, indinv, indinv_len, ncouls, g);
    if (igp_of[g] == -2) return -2;
  }
  const cd* aqsm = reinterpret_cast<const cd*>(aqsmtemp);
  const cd* aqsn = reinterpret_cast<const cd*>(aqsntemp);
  const cd* ieps = reinterpret_cast<const cd*>(I_eps_array);
  const cd* wtil = reinterpret_cast<const cd*>(wtilde_array);
  const size_t nc = static_cast<size_t>(ncouls);
  if (nthreads <= 0) nthreads = omp_get_max_threads();

  CDD ach_total[3], asx_total[3], stat_total;
  std::vector<CDD> sch_c(static_cast<size_t>(ngpown) * 3), ssx_c(static_cast<size_t>(ngpown) * 3);
  std::vector<CDD> stat_c(ngpown);
  for (int n1 = band_begin; n1 < band_end; ++n1) {
    const bool flag_occ = n1 < nvband;
    const cd* nrow = aqsn + n1 * nc;
    const cd* mrow = aqsm + n1 * nc;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
      const int igp = igp_of[my_igp];
      CDD sch[3], ssx[3], stat;
      if (igp >= 0) {
        const cd* wrow = wtil + my_igp * nc;
        const cd* erow = ieps + my_igp * nc;
        const int igmax = igp;
        // static remainder, reduce_achstemp (gppKerSeq.cpp:27-70)
        if (achstemp) {
          const cd v1 = std::conj(mrow[igp]);
          const cd v2 = nrow[igp];
          for (int ig = 0; ig < igmax; ++ig) {
            const cd schs = -erow[ig];
            const cd matngmatmgp = nrow[ig] * v1;
            const cd matngpmatmg = std::conj(mrow[ig]) * v2;
            stat.add(matngmatmgp * schs + matngpmatmg * std::conj(schs));
          }
          const cd schs = -erow[igp];
          if (std::abs(schs) > kTo1) stat.add(nrow[igp] * v1 * schs);
        }
        const cd mygpvar1 = std::conj(mrow[igp]);
        const cd mygpvar2 = mrow[igp];
        for (int iw = 0; iw < 3; ++iw) {
          if (flag_occ) {
            half_occ(wx[iw], igmax, igp, wrow, erow, nrow, mrow, mygpvar1, mygpvar2, ssx[iw],
                     sch[iw]);
          } else {
            for (int igbeg = 0; igbeg < igmax; igbeg += kIgBlk) {
              const int igend = std::min(igbeg + kIgBlk - 1, igmax);
              half_block(igbeg, igend, igmax, wx[iw], wrow, erow, nrow, mrow, mygpvar1,
                         mygpvar2, sch[iw]);
            }
          }
        }
      }
      for (int iw = 0; iw < 3; ++iw) {
        sch_c[my_igp * 3 + iw] = sch[iw];
        ssx_c[my_igp * 3 + iw] = ssx[iw];
      }
      stat_c[my_igp] = stat;
    }
    // epilogue (gppKerSeq.cpp:473-488): sch_array = 0.5 scht, times vcoul[igp]
    CDD band[3];
    for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
      const int igp = igp_of[my_igp];
      const double v = igp >= 0 ? vcoul[igp] : 0.0;
      for (int iw = 0; iw < 3; ++iw) {
        const cd s = 0.5 * sch_c[my_igp * 3 + iw].value();
        const cd x = ssx_c[my_igp * 3 + iw].value();
        band[iw].add(s * v);
        if (flag_occ) asx_total[iw].add(x * occ * v);
        if (col_sch) {
          const int64_t o = (static_cast<int64_t>(n1) * ngpown + my_igp) * 3 + iw;
          col_sch[2 * o] = s.real();
          col_sch[2 * o + 1] = s.imag();
          if (col_ssx) {
            col_ssx[2 * o] = x.real();
            col_ssx[2 * o + 1] = x.imag();
          }
        }
      }
      if (achstemp) stat_total.add(stat_c[my_igp].value() * v * 0.5);
    }
    for (int iw = 0; iw < 3; ++iw) ach_total[iw].add(band[iw]);
    if (acht_n1_loc) {
      const cd v = band[2].value();
      acht_n1_loc[2 * n1] = v.real();
      acht_n1_loc[2 * n1 + 1] = v.imag();
    }
  }
  for (int iw = 0; iw < 3; ++iw) {
    const cd a = ach_total[iw].value(), s = asx_total[iw].value();
    achtemp[2 * iw] = a.real();
    achtemp[2 * iw + 1] = a.imag();
    asxtemp[2 * iw] = s.real();
    asxtemp[2 * iw + 1] = s.imag();
  }
  if (achstemp) {
    const cd s = stat_total.value();
    achstemp[0] = s.real();
    achstemp[1] = s.imag();
  }
  return 0;
}

}  // extern "C"
