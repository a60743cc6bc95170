// CPU oracle for the sigma GPP / FF hot path.  TEST INFRASTRUCTURE ONLY:
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it;
// the product library never links or calls it.
//
// It restates the reference algorithm per term with std::complex<double>,
// in the reference's operation order, and sums the terms in a fixed order
// with double-double (compensated) accumulators, so its result does not
// depend on the thread count and is more accurate than the reference's own
// OpenMP sums (which reorder from run to run, schedule(dynamic)).
//
// Sources restated (paths relative to the reference project):
//   term of the non-occupied bands   BGW-Kernels/gppKer.cpp:394-407
//   term of the occupied bands       BGW-Kernels/gppKer.cpp:19-65, 145-158
//   per-igp epilogue and reduction   BGW-Kernels/gppKer.cpp:411, 416-424, 431-439
//   index mapping                    BGW-Kernels/gppKer.cpp:322-328
//   FF schDt contraction             ffkernel.deslippe.best.f90:402-418 (commented
//                                    zgemm + conj(aqsm) reduction), C layouts of
//                                    FFKer_cori/ffKernel.cpp:366,386,434
//
// A second GPP entry, oracle_gpp_port, keeps the reference's loop structure
// and plain double sums (n1 outer, OpenMP dynamic over my_igp, 512-wide ig
// blocks) and is the CPU baseline that bench.py times on hosts where the
// unmodified reference binary cannot be built.
//
// Build with -ffp-contract=off so x86 and aarch64 hosts round every term alike.

#include <complex>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

using cd = std::complex<double>;

constexpr double kTo1 = 1e-6;
constexpr double kLimitOne = 1.0 / (kTo1 * 4.0);
constexpr double kLimitTwo = 0.5 * 0.5;

enum {
  kOk = 0,
  kErrShape = -1,
  kErrIndex = -2,
  kErrNull = -6,
};

// ---- double-double accumulation (Dekker / Knuth error-free transforms) ----
struct DD {
  double hi = 0.0, lo = 0.0;
};

inline void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double bv = s - a;
  e = (a - (s - bv)) + (b - bv);
}

inline void dd_add(DD& x, double y) {
  double s, e;
  two_sum(x.hi, y, s, e);
  e += x.lo;
  x.hi = s + e;
  x.lo = e - (x.hi - s);
}

inline void dd_add(DD& x, const DD& y) {
  double s, e;
  two_sum(x.hi, y.hi, s, e);
  e += x.lo + y.lo;
  x.hi = s + e;
  x.lo = e - (x.hi - s);
}

inline DD dd_mul(const DD& x, double y) {
  double p = x.hi * y;
  double e = std::fma(x.hi, y, -p) + x.lo * y;
  DD r;
  r.hi = p + e;
  r.lo = e - (r.hi - p);
  return r;
}

struct CDD {
  DD re, im;
  void add(const cd& v) { dd_add(re, v.real()); dd_add(im, v.imag()); }
  void add(const CDD& v) { dd_add(re, v.re); dd_add(im, v.im); }
  CDD scaled(double s) const { CDD r; r.re = dd_mul(re, s); r.im = dd_mul(im, s); return r; }
  cd value() const { return cd(re.hi + re.lo, im.hi + im.lo); }
};

// ---- per-term arithmetic, reference operation order ----

// Non-occupied band term (BGW-Kernels/gppKer.cpp:396-407).  Returns scha and
// whether the pole guard lets it into the sum.
inline cd term_unocc(double wxt, const cd& wt, const cd& mygpvar1, const cd& aqsn,
                     const cd& ieps, bool& keep) {
  cd wdiff = wxt - wt;
  cd cden = wdiff;
  double rden = std::real(cden * std::conj(cden));
  rden = 1 / rden;
  cd delw = wt * std::conj(cden) * rden;
  double delwr = std::real(delw * std::conj(delw));
  double wdiffr = std::real(wdiff * std::conj(wdiff));
  cd scha = mygpvar1 * aqsn * delw * ieps;
  keep = (wdiffr > kLimitTwo) && (delwr < kLimitOne);
  return scha;
}

// Occupied band term: ssxt_scht_solver as flagOCC_solver drives it
// (BGW-Kernels/gppKer.cpp:19-65, 147-155).  Writes ssxa and scha.
inline void term_occ(double wxt, const cd& wt, const cd& mygpvar1, const cd& aqsn,
                     const cd& ieps, cd& ssxa, cd& scha) {
  cd wtilde2 = wt * wt;  // std::pow(wtilde, 2) in libstdc++ is 1 * (w * w)
  cd omega2 = wtilde2 * ieps;
  cd matngmatmgp = aqsn * mygpvar1;

  cd wdiff = wxt - wt;
  cd cden = wdiff;
  double rden = 1 / std::real(cden * std::conj(cden));
  cd delw = wt * std::conj(cden) * rden;
  double delwr = std::real(delw * std::conj(delw));
  double wdiffr = std::real(wdiff * std::conj(wdiff));
  cd sch, ssx;
  if ((wdiffr > kLimitTwo) && (delwr < kLimitOne)) {
    sch = delw * ieps;
    cden = cd(wxt * wxt, 0.0);
    rden = std::real(cden * std::conj(cden));
    rden = 1.00 / rden;
    ssx = omega2 * std::conj(cden) * rden;
  } else if (delwr > kTo1) {
    sch = cd(0.0, 0.0);
    cden = 4.00 * wtilde2 * (delw + 0.50);
    rden = std::real(cden * std::conj(cden));
    rden = 1.00 / rden;
    ssx = -omega2 * std::conj(cden) * rden * delw;
  } else {
    sch = cd(0.0, 0.0);
    ssx = cd(0.0, 0.0);
  }
  // the ssxcutoff test of :60-61 compares abs(wxt) < 0 and never fires
  ssxa = matngmatmgp * ssx;
  scha = matngmatmgp * sch;
}

// igp for my_igp (BGW-Kernels/gppKer.cpp:322-328).  Returns -1 for a skipped
// column, -2 for an index the reference would read out of bounds.
inline int map_igp(const int* inv_igp_index, const int* indinv, int indinv_len, int ncouls,
                   int my_igp) {
  int indigp = inv_igp_index[my_igp];
  if (indigp < 0 || indigp > ncouls) return -2;
  int igp;
  if (indigp == ncouls) {
    igp = ncouls - 1;
  } else {
    if (indigp >= indinv_len) return -2;
    igp = indinv[indigp];
  }
  if (igp > ncouls || igp < 0) return -1;
  if (igp == ncouls) return -2;  // the reference would read aqsmtemp/vcoul past the row
  return igp;
}

}  // namespace

extern "C" {

// Compensated GPP oracle.  Arrays are interleaved complex128 (re, im) as in
// std::complex<double>.  wx_array holds nw = nend - nstart frequencies per
// band with stride wx_band_stride (0: one set shared by every band, the
// mini-app's case).  Bands [band_begin, band_end) are summed; achtemp and
// asxtemp receive their sums over those bands, acht_n1_loc[n1] is written
// for those bands only.  Returns 0 or a negative error code.
int oracle_gpp(int number_bands, int nvband, int ncouls, int ngpown, int nstart, int nend,
               const int* inv_igp_index, const int* indinv, int indinv_len,
               const double* wx_array, int wx_band_stride, double occ,
               const double* aqsmtemp, const double* aqsntemp, const double* I_eps_array,
               const double* wtilde_array, const double* vcoul, double* achtemp,
               double* asxtemp, double* acht_n1_loc, int band_begin, int band_end,
               int nthreads) {
  if (!inv_igp_index || !indinv || !wx_array || !aqsmtemp || !aqsntemp || !I_eps_array ||
      !wtilde_array || !vcoul || !achtemp || !asxtemp)
    return kErrNull;
  const int nw = nend - nstart;
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0 || nw != 3 || nstart != 0 ||
      nvband < 0 || band_begin < 0 || band_end > number_bands || band_begin > band_end)
    return kErrShape;
  std::vector<int> igp_of(ngpown);
  for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
    int g = map_igp(inv_igp_index, indinv, indinv_len, ncouls, my_igp);
    if (g == -2) return kErrIndex;
    igp_of[my_igp] = g;
  }
  const cd* aqsm = reinterpret_cast<const cd*>(aqsmtemp);
  const cd* aqsn = reinterpret_cast<const cd*>(aqsntemp);
  const cd* ieps = reinterpret_cast<const cd*>(I_eps_array);
  const cd* wtil = reinterpret_cast<const cd*>(wtilde_array);
  const size_t nc = static_cast<size_t>(ncouls);
  if (nthreads <= 0) nthreads = omp_get_max_threads();

  CDD ach_total[3], asx_total[3];
  // per (my_igp) results of one band, reduced in my_igp order afterwards
  std::vector<CDD> sch_igp(static_cast<size_t>(ngpown) * 3), ssx_igp(static_cast<size_t>(ngpown) * 3);

  for (int n1 = band_begin; n1 < band_end; ++n1) {
    const bool flag_occ = n1 < nvband;
    const double* wx = wx_array + static_cast<size_t>(wx_band_stride) * n1;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
      const int igp = igp_of[my_igp];
      CDD sch[3], ssx[3];
      if (igp >= 0) {
        const cd mygpvar1 = std::conj(aqsm[n1 * nc + igp]);
        const cd* wrow = wtil + my_igp * nc;
        const cd* erow = ieps + my_igp * nc;
        const cd* nrow = aqsn + n1 * nc;
        for (int iw = 0; iw < 3; ++iw) {
          const double wxt = wx[iw];
          for (size_t ig = 0; ig < nc; ++ig) {
            if (flag_occ) {
              cd ssxa, scha;
              term_occ(wxt, wrow[ig], mygpvar1, nrow[ig], erow[ig], ssxa, scha);
              ssx[iw].add(ssxa);
              sch[iw].add(scha);
            } else {
              bool keep;
              cd scha = term_unocc(wxt, wrow[ig], mygpvar1, nrow[ig], erow[ig], keep);
              if (keep) sch[iw].add(scha);
            }
          }
        }
      }
      for (int iw = 0; iw < 3; ++iw) {
        // sch_array[iw] += 0.5 * scht; achtemp += sch_array * vcoul[igp]
        const double v = igp >= 0 ? vcoul[igp] : 0.0;
        sch_igp[my_igp * 3 + iw] = sch[iw].scaled(0.5).scaled(v);
        ssx_igp[my_igp * 3 + iw] = ssx[iw].scaled(occ).scaled(v);
      }
    }
    CDD band[3];
    for (int my_igp = 0; my_igp < ngpown; ++my_igp)
      for (int iw = 0; iw < 3; ++iw) {
        band[iw].add(sch_igp[my_igp * 3 + iw]);
        if (flag_occ) asx_total[iw].add(ssx_igp[my_igp * 3 + iw]);
      }
    for (int iw = 0; iw < 3; ++iw) ach_total[iw].add(band[iw]);
    if (acht_n1_loc) {
      cd v = band[2].value();
      acht_n1_loc[2 * n1] = v.real();
      acht_n1_loc[2 * n1 + 1] = v.imag();
    }
  }
  for (int iw = 0; iw < 3; ++iw) {
    cd a = ach_total[iw].value(), s = asx_total[iw].value();
    achtemp[2 * iw] = a.real();
    achtemp[2 * iw + 1] = a.imag();
    asxtemp[2 * iw] = s.real();
    asxtemp[2 * iw + 1] = s.imag();
  }
  return kOk;
}

// The reference's loop nest with plain double sums, for timing on the host's
// cores: n1 outer, `omp parallel for schedule(dynamic)` over my_igp, ig in
// 512-wide blocks, per-thread partial arrays reduced at the end
// (BGW-Kernels/gppKer.cpp:303-439).  Its last digits vary from run to run,
// as the reference's do.  reduce_achstemp (:308), whose result the reference
// discards, is not run.
int oracle_gpp_port(int number_bands, int nvband, int ncouls, int ngpown, int nstart, int nend,
                    const int* inv_igp_index, const int* indinv, int indinv_len,
                    const double* wx_array, int wx_band_stride, double occ,
                    const double* aqsmtemp, const double* aqsntemp, const double* I_eps_array,
                    const double* wtilde_array, const double* vcoul, double* achtemp,
                    double* asxtemp, double* acht_n1_loc, int band_begin, int band_end,
                    int nthreads) {
  if (!inv_igp_index || !indinv || !wx_array || !aqsmtemp || !aqsntemp || !I_eps_array ||
      !wtilde_array || !vcoul || !achtemp || !asxtemp)
    return kErrNull;
  const int nw = nend - nstart;
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0 || nw != 3 || nstart != 0 ||
      band_begin < 0 || band_end > number_bands || band_begin > band_end)
    return kErrShape;
  std::vector<int> igp_of(ngpown);
  for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
    int g = map_igp(inv_igp_index, indinv, indinv_len, ncouls, my_igp);
    if (g == -2) return kErrIndex;
    igp_of[my_igp] = g;
  }
  const cd* aqsm = reinterpret_cast<const cd*>(aqsmtemp);
  const cd* aqsn = reinterpret_cast<const cd*>(aqsntemp);
  const cd* ieps = reinterpret_cast<const cd*>(I_eps_array);
  const cd* wtil = reinterpret_cast<const cd*>(wtilde_array);
  const size_t nc = static_cast<size_t>(ncouls);
  if (nthreads <= 0) nthreads = omp_get_max_threads();

  std::vector<cd> ach_thr(static_cast<size_t>(nthreads) * 3, cd(0, 0));
  std::vector<cd> n1_thr(static_cast<size_t>(nthreads) * number_bands, cd(0, 0));
  cd asx[3] = {cd(0, 0), cd(0, 0), cd(0, 0)};
  const int igblk = 512;

  for (int n1 = band_begin; n1 < band_end; ++n1) {
    const bool flag_occ = n1 < nvband;
    const double* wx = wx_array + static_cast<size_t>(wx_band_stride) * n1;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
    for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
      const int tid = omp_get_thread_num();
      const int igp = igp_of[my_igp];
      if (igp < 0) continue;
      cd ssx_array[3] = {cd(0, 0), cd(0, 0), cd(0, 0)};
      cd sch_array[3] = {cd(0, 0), cd(0, 0), cd(0, 0)};
      const cd mygpvar1 = std::conj(aqsm[n1 * nc + igp]);
      const cd* wrow = wtil + my_igp * nc;
      const cd* erow = ieps + my_igp * nc;
      const cd* nrow = aqsn + n1 * nc;
      if (flag_occ) {
        for (int iw = 0; iw < 3; ++iw) {
          cd scht(0, 0), ssxt(0, 0);
          for (size_t ig = 0; ig < nc; ++ig) {
            cd ssxa, scha;
            term_occ(wx[iw], wrow[ig], mygpvar1, nrow[ig], erow[ig], ssxa, scha);
            ssxt += ssxa;
            scht += scha;
          }
          ssx_array[iw] += ssxt;
          sch_array[iw] += 0.5 * scht;
        }
      } else {
        for (size_t igbeg = 0; igbeg < nc; igbeg += igblk) {
          const size_t igend = std::min(igbeg + igblk, nc);
          for (int iw = 0; iw < 3; ++iw) {
            cd scht(0, 0);
            for (size_t ig = igbeg; ig < igend; ++ig) {
              bool keep;
              cd scha = term_unocc(wx[iw], wrow[ig], mygpvar1, nrow[ig], erow[ig], keep);
              if (keep) scht += scha;
            }
            sch_array[iw] += 0.5 * scht;
          }
        }
      }
      if (flag_occ)
        for (int iw = 0; iw < 3; ++iw) {
#pragma omp critical
          asx[iw] += ssx_array[iw] * occ * vcoul[igp];
        }
      for (int iw = 0; iw < 3; ++iw) ach_thr[tid * 3 + iw] += sch_array[iw] * vcoul[igp];
      n1_thr[static_cast<size_t>(tid) * number_bands + n1] += sch_array[2] * vcoul[igp];
    }
  }
  for (int iw = 0; iw < 3; ++iw) {
    cd a(0, 0);
    for (int t = 0; t < nthreads; ++t) a += ach_thr[t * 3 + iw];
    achtemp[2 * iw] = a.real();
    achtemp[2 * iw + 1] = a.imag();
    asxtemp[2 * iw] = asx[iw].real();
    asxtemp[2 * iw + 1] = asx[iw].imag();
  }
  if (acht_n1_loc)
    for (int n1 = band_begin; n1 < band_end; ++n1) {
      cd a(0, 0);
      for (int t = 0; t < nthreads; ++t) a += n1_thr[static_cast<size_t>(t) * number_bands + n1];
      acht_n1_loc[2 * n1] = a.real();
      acht_n1_loc[2 * n1 + 1] = a.imag();
    }
  return kOk;
}

// Per-(n1, my_igp, iw) sums of one band range, for fine-grained checks:
// out_sch / out_ssx are [band_end - band_begin][ngpown][3] complex and hold
// sch_array[iw] (0.5 * scht, before vcoul) and ssx_array[iw] of each column.
// Skipped columns read zero.
int oracle_gpp_columns(int number_bands, int nvband, int ncouls, int ngpown,
                       const int* inv_igp_index, const int* indinv, int indinv_len,
                       const double* wx_array, int wx_band_stride, const double* aqsmtemp,
                       const double* aqsntemp, const double* I_eps_array,
                       const double* wtilde_array, double* out_sch, double* out_ssx,
                       int band_begin, int band_end, int nthreads) {
  if (band_begin < 0 || band_end > number_bands || band_begin > band_end) return kErrShape;
  std::vector<int> igp_of(ngpown);
  for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
    int g = map_igp(inv_igp_index, indinv, indinv_len, ncouls, my_igp);
    if (g == -2) return kErrIndex;
    igp_of[my_igp] = g;
  }
  const cd* aqsm = reinterpret_cast<const cd*>(aqsmtemp);
  const cd* aqsn = reinterpret_cast<const cd*>(aqsntemp);
  const cd* ieps = reinterpret_cast<const cd*>(I_eps_array);
  const cd* wtil = reinterpret_cast<const cd*>(wtilde_array);
  const size_t nc = static_cast<size_t>(ncouls);
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  const int nbr = band_end - band_begin;
#pragma omp parallel for collapse(2) schedule(dynamic, 4) num_threads(nthreads)
  for (int b = 0; b < nbr; ++b)
    for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
      const int n1 = band_begin + b;
      const int igp = igp_of[my_igp];
      const bool flag_occ = n1 < nvband;
      const double* wx = wx_array + static_cast<size_t>(wx_band_stride) * n1;
      CDD sch[3], ssx[3];
      if (igp >= 0) {
        const cd mygpvar1 = std::conj(aqsm[n1 * nc + igp]);
        for (int iw = 0; iw < 3; ++iw)
          for (size_t ig = 0; ig < nc; ++ig) {
            const cd wt = wtil[my_igp * nc + ig], ie = ieps[my_igp * nc + ig],
                     an = aqsn[n1 * nc + ig];
            if (flag_occ) {
              cd ssxa, scha;
              term_occ(wx[iw], wt, mygpvar1, an, ie, ssxa, scha);
              ssx[iw].add(ssxa);
              sch[iw].add(scha);
            } else {
              bool keep;
              cd scha = term_unocc(wx[iw], wt, mygpvar1, an, ie, keep);
              if (keep) sch[iw].add(scha);
            }
          }
      }
      const size_t o = (static_cast<size_t>(b) * ngpown + my_igp) * 3;
      for (int iw = 0; iw < 3; ++iw) {
        cd s = sch[iw].scaled(0.5).value(), x = ssx[iw].value();
        out_sch[2 * (o + iw)] = s.real();
        out_sch[2 * (o + iw) + 1] = s.imag();
        out_ssx[2 * (o + iw)] = x.real();
        out_ssx[2 * (o + iw) + 1] = x.imag();
      }
    }
  return kOk;
}

// Sum of squared term magnitudes of every output: ach_abs2[iw] = sum over
// the terms that enter achtemp[iw] of |scha * 0.5 * vcoul[igp]|^2, and
// asx_abs2[iw] likewise for asxtemp[iw] (|ssxa * occ * vcoul[igp]|^2).  A
// method whose per-term relative error is e (independent, rms) misses the
// exact sum by about e * sqrt(abs2); sqrt(abs2) / |sum| is the output's
// cancellation factor.  Same terms and guard as oracle_gpp; only bands
// [band_begin, band_end) are summed (a band sample, for large instances).
int oracle_gpp_abs2(int number_bands, int nvband, int ncouls, int ngpown,
                    const int* inv_igp_index, const int* indinv, int indinv_len,
                    const double* wx_array, int wx_band_stride, double occ,
                    const double* aqsmtemp, const double* aqsntemp, const double* I_eps_array,
                    const double* wtilde_array, const double* vcoul, double* ach_abs2,
                    double* asx_abs2, int band_begin, int band_end, int nthreads) {
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0 || nvband < 0) return kErrShape;
  if (band_begin < 0 || band_end > number_bands || band_begin > band_end) return kErrShape;
  std::vector<int> igp_of(ngpown);
  for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
    int g = map_igp(inv_igp_index, indinv, indinv_len, ncouls, my_igp);
    if (g == -2) return kErrIndex;
    igp_of[my_igp] = g;
  }
  const cd* aqsm = reinterpret_cast<const cd*>(aqsmtemp);
  const cd* aqsn = reinterpret_cast<const cd*>(aqsntemp);
  const cd* ieps = reinterpret_cast<const cd*>(I_eps_array);
  const cd* wtil = reinterpret_cast<const cd*>(wtilde_array);
  const size_t nc = static_cast<size_t>(ncouls);
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  std::vector<double> per(static_cast<size_t>(ngpown) * 6, 0.0);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
  for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
    const int igp = igp_of[my_igp];
    if (igp < 0) continue;
    double s[6] = {0, 0, 0, 0, 0, 0};
    const double v = vcoul[igp];
    for (int n1 = band_begin; n1 < band_end; ++n1) {
      const cd mygpvar1 = std::conj(aqsm[n1 * nc + igp]);
      const double* wx = wx_array + static_cast<size_t>(wx_band_stride) * n1;
      for (int iw = 0; iw < 3; ++iw)
        for (size_t ig = 0; ig < nc; ++ig) {
          const cd wt = wtil[my_igp * nc + ig], ie = ieps[my_igp * nc + ig], an = aqsn[n1 * nc + ig];
          if (n1 < nvband) {
            cd ssxa, scha;
            term_occ(wx[iw], wt, mygpvar1, an, ie, ssxa, scha);
            s[iw] += std::norm(scha * (0.5 * v));
            s[3 + iw] += std::norm(ssxa * (occ * v));
          } else {
            bool keep;
            cd scha = term_unocc(wx[iw], wt, mygpvar1, an, ie, keep);
            if (keep) s[iw] += std::norm(scha * (0.5 * v));
          }
        }
    }
    for (int k = 0; k < 6; ++k) per[static_cast<size_t>(my_igp) * 6 + k] = s[k];
  }
  for (int k = 0; k < 3; ++k) ach_abs2[k] = asx_abs2[k] = 0.0;
  for (int my_igp = 0; my_igp < ngpown; ++my_igp)
    for (int k = 0; k < 3; ++k) {
      ach_abs2[k] += per[static_cast<size_t>(my_igp) * 6 + k];
      asx_abs2[k] += per[static_cast<size_t>(my_igp) * 6 + 3 + k];
    }
  return kOk;
}

// Static remainder of the GPP sum, Fortran formula
// (gppkernel.deslippe.09.30.2014.f90:195-228; the C++ reduce_achstemp,
// BGW-Kernels/gppKer.cpp:67-128, is not a usable statement of it):
//   schstemp = sum_ig -aqsn[n1][ig] * I_eps[my_igp][ig] * conj(aqsm[n1][igp])
//   achstemp += schstemp * vcoul[igp] * 0.5
// in that operation order, index map and skipped columns as oracle_gpp,
// double-double sums.  out_n1 (complex[number_bands], may be NULL) receives
// each band's sum, out (complex[1]) the total.
int oracle_gpp_achstemp(int number_bands, int ncouls, int ngpown, const int* inv_igp_index,
                        const int* indinv, int indinv_len, const double* aqsmtemp,
                        const double* aqsntemp, const double* I_eps_array, const double* vcoul,
                        double* out, double* out_n1, int nthreads) {
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0) return kErrShape;
  std::vector<int> igp_of(ngpown);
  for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
    int g = map_igp(inv_igp_index, indinv, indinv_len, ncouls, my_igp);
    if (g == -2) return kErrIndex;
    igp_of[my_igp] = g;
  }
  const cd* aqsm = reinterpret_cast<const cd*>(aqsmtemp);
  const cd* aqsn = reinterpret_cast<const cd*>(aqsntemp);
  const cd* ieps = reinterpret_cast<const cd*>(I_eps_array);
  const size_t nc = static_cast<size_t>(ncouls);
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  std::vector<CDD> band(number_bands);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int n1 = 0; n1 < number_bands; ++n1) {
    CDD acc;
    for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
      const int igp = igp_of[my_igp];
      if (igp < 0) continue;
      const cd mygpvar1 = std::conj(aqsm[n1 * nc + igp]);
      CDD sch;
      for (size_t ig = 0; ig < nc; ++ig) sch.add(-(aqsn[n1 * nc + ig] * ieps[my_igp * nc + ig] * mygpvar1));
      acc.add(sch.scaled(vcoul[igp]).scaled(0.5));
    }
    band[n1] = acc;
  }
  CDD total;
  for (int n1 = 0; n1 < number_bands; ++n1) {
    total.add(band[n1]);
    if (out_n1) {
      cd v = band[n1].value();
      out_n1[2 * n1] = v.real();
      out_n1[2 * n1 + 1] = v.imag();
    }
  }
  cd t = total.value();
  out[0] = t.real();
  out[1] = t.imag();
  return kOk;
}

// FF schDt contraction for a list of (n1, ifreq) entries:
//   schDt[n1][ifreq] = sum_my_igp (sum_ig I_epsR[ifreq][my_igp][ig] * aqsn[n1][ig])
//                      * conj(aqsm[n1][igp(my_igp)])
// (ffkernel.deslippe.best.f90:404-418; igp = indinv[inv_igp_index[my_igp]]
// with no clamp, as FFKer_cori/ffKernel.cpp:114-115 maps it).  out is
// complex[n_entries].  Double-double sums.
int oracle_ff_schdt(int number_bands, int ncouls, int ngpown, int nfreq,
                    const int* inv_igp_index, const int* indinv, const double* I_epsR,
                    const double* aqsntemp, const double* aqsmtemp, int n_entries,
                    const int* entry_n1, const int* entry_ifreq, double* out, int nthreads) {
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0 || nfreq <= 0) return kErrShape;
  std::vector<int> igp_of(ngpown);
  for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
    int ind = inv_igp_index[my_igp];
    if (ind < 0 || ind >= ncouls) return kErrIndex;
    int g = indinv[ind];
    if (g < 0 || g >= ncouls) return kErrIndex;
    igp_of[my_igp] = g;
  }
  for (int e = 0; e < n_entries; ++e)
    if (entry_n1[e] < 0 || entry_n1[e] >= number_bands || entry_ifreq[e] < 0 ||
        entry_ifreq[e] >= nfreq)
      return kErrShape;
  const cd* epsr = reinterpret_cast<const cd*>(I_epsR);
  const cd* aqsn = reinterpret_cast<const cd*>(aqsntemp);
  const cd* aqsm = reinterpret_cast<const cd*>(aqsmtemp);
  const size_t nc = static_cast<size_t>(ncouls);
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
  for (int e = 0; e < n_entries; ++e) {
    const int n1 = entry_n1[e], f = entry_ifreq[e];
    CDD acc;
    for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
      CDD tz;
      const cd* row = epsr + (static_cast<size_t>(f) * ngpown + my_igp) * nc;
      const cd* an = aqsn + n1 * nc;
      for (size_t ig = 0; ig < nc; ++ig) {
        // exact products of the parts, summed in double-double
        const double a = row[ig].real(), b = row[ig].imag(), c = an[ig].real(), d = an[ig].imag();
        double p, q;
        p = a * c; q = std::fma(a, c, -p); dd_add(tz.re, p); dd_add(tz.re, q);
        p = -b * d; q = std::fma(-b, d, -p); dd_add(tz.re, p); dd_add(tz.re, q);
        p = a * d; q = std::fma(a, d, -p); dd_add(tz.im, p); dd_add(tz.im, q);
        p = b * c; q = std::fma(b, c, -p); dd_add(tz.im, p); dd_add(tz.im, q);
      }
      const cd m = std::conj(aqsm[n1 * nc + igp_of[my_igp]]);
      // tz * m in double-double: (tr + i ti)(mr + i mi)
      DD t1 = dd_mul(tz.re, m.real()), t2 = dd_mul(tz.im, m.imag());
      DD t3 = dd_mul(tz.re, m.imag()), t4 = dd_mul(tz.im, m.real());
      t2.hi = -t2.hi; t2.lo = -t2.lo;
      dd_add(acc.re, t1); dd_add(acc.re, t2);
      dd_add(acc.im, t3); dd_add(acc.im, t4);
    }
    cd v = acc.value();
    out[2 * e] = v.real();
    out[2 * e + 1] = v.imag();
  }
  return kOk;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Full-frequency sigma: the band loop of ffkernel.deslippe.best.f90
// (:201-626) around the schDt contraction, 0-based, in the C layouts of
// FFKer_cori/ffKernel.cpp (I_epsR / I_epsA [nfreq][ngpown][ncouls],
// aqsm / aqsn [number_bands][ncouls], schDt_matrix [number_bands][nfreq]).
// Outputs (complex): achsDtemp[1], asxDtemp, achDtemp, achDtemp_cor,
// achDtemp_corb, ach2Dtemp [nfreqeval] each, overwritten.
//   static CH (:236-254)          achsDtemp
//   SX, occupied bands (:279-389) asxDtemp
//   CH from schDt (:459-521)      achDtemp (sigma1), achDtemp_corb (sigma3),
//                                 ach2Dtemp (sigma2), achDtemp_cor (sigma4)
//   delta-function terms (:530-613) ach2Dtemp, achDtemp_cor
// with wx = freqevalmin - ekq[n1] + iw * freqevalstep.  schDt_matrix is an
// input, as achDtemp_Kernel takes it (FFKer_cori/ffKernel.cpp:155); the live
// Fortran zeroes it (:395) because its contraction is commented out.
// Columns whose igp falls outside [0, ncouls) are skipped as the Fortran
// skips them.  Sums in double-double, each band's terms in the Fortran
// operation order.

namespace {

// Last grid interval [g[k], g[k+1]) holding w, k in 0..nfreq-2; nfreq-2 when
// none does (both searches of the Fortran end there: :288-311, :536-545).
int ff_interval(double w, const double* grid, int nfreq) {
  int k = -1;
  for (int j = 0; j < nfreq - 1; ++j)
    if (w >= grid[j] && w < grid[j + 1]) k = j;
  return k < 0 ? nfreq - 2 : k;
}

// sum_{my_igp valid} vcoul[igp] * sum_ig aqsn[n1][ig] conj(aqsm[n1][igp])
//     * (f1 X1[my_igp][ig] + f2 X2[my_igp][ig])   (:339-346, :582-589)
// with X = a - b when b is given (I_epsR - I_epsA), the element combination
// and product order of the Fortran.
cd ff_weighted_pair(int n1, int ncouls, int ngpown, const std::vector<int>& igp_of, const cd* aqsm,
                    const cd* aqsn, const double* vcoul, const cd* a1, const cd* b1, const cd* a2,
                    const cd* b2, double f1, double f2, double scale) {
  const size_t nc = static_cast<size_t>(ncouls);
  CDD tot;
  for (int g = 0; g < ngpown; ++g) {
    const int igp = igp_of[g];
    if (igp < 0) continue;
    CDD t;
    const cd m = std::conj(aqsm[n1 * nc + igp]);
    for (size_t ig = 0; ig < nc; ++ig) {
      const size_t o = static_cast<size_t>(g) * nc + ig;
      cd x;
      if (b1)
        x = (a1[o] - b1[o]) * f1 + (a2[o] - b2[o]) * f2;
      else
        x = a1[o] * f1 + a2[o] * f2;
      if (scale != 1.0) x = scale * x;
      t.add(aqsn[n1 * nc + ig] * m * x);
    }
    tot.add(t.scaled(vcoul[igp]));
  }
  return tot.value();
}

}  // namespace

extern "C" int oracle_ff_sigma(int number_bands, int nvband, int ncouls, int ngpown, int nfreq,
                               int nfreqeval, const int* inv_igp_index, const int* indinv,
                               const double* aqsmtemp, const double* aqsntemp, const double* I_epsR,
                               const double* I_epsA, const double* vcoul, const double* ekq,
                               const double* dFreqGrid, const double* dFreqBrd, const double* pref,
                               double pref_zb, double freqevalmin, double freqevalstep, double occ,
                               const double* schDt_matrix, double* achsDtemp, double* asxDtemp,
                               double* achDtemp, double* achDtemp_cor, double* achDtemp_corb,
                               double* ach2Dtemp, int nthreads) {
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0 || nfreq < 2 || nfreqeval <= 0 || nvband < 0)
    return kErrShape;
  std::vector<int> igp_of(ngpown);
  for (int g = 0; g < ngpown; ++g) {
    const int ind = inv_igp_index[g];
    if (ind < 0 || ind >= ncouls) return kErrIndex;
    const int igp = indinv[ind];
    igp_of[g] = (igp < 0 || igp >= ncouls) ? -1 : igp;
  }
  const cd* aqsm = reinterpret_cast<const cd*>(aqsmtemp);
  const cd* aqsn = reinterpret_cast<const cd*>(aqsntemp);
  const cd* epsR = reinterpret_cast<const cd*>(I_epsR);
  const cd* epsA = reinterpret_cast<const cd*>(I_epsA);
  const cd* brd = reinterpret_cast<const cd*>(dFreqBrd);
  const cd* sdt = reinterpret_cast<const cd*>(schDt_matrix);
  const size_t nc = static_cast<size_t>(ncouls);
  const size_t slab = static_cast<size_t>(ngpown) * nc;
  const cd I(0.0, 1.0);
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  const int ne = nfreqeval;
  // per band: [0] achs, then 5 arrays of ne: asx, ach, ach_cor, ach_corb, ach2
  std::vector<CDD> per(static_cast<size_t>(number_bands) * (1 + 5 * ne));
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int n1 = 0; n1 < number_bands; ++n1) {
    CDD* r = &per[static_cast<size_t>(n1) * (1 + 5 * ne)];
    CDD* asx = r + 1;
    CDD* schDi = asx + ne;
    CDD* schDi_cor = schDi + ne;
    CDD* schDi_corb = schDi_cor + ne;
    CDD* sch2Di = schDi_corb + ne;
    const bool flag_occ = n1 < nvband;
    // static CH (:240-253)
    for (int g = 0; g < ngpown; ++g) {
      const int igp = igp_of[g];
      if (igp < 0) continue;
      CDD t;
      const cd m = std::conj(aqsm[n1 * nc + igp]);
      for (size_t ig = 0; ig < nc; ++ig)
        t.add(-(aqsn[n1 * nc + ig] * m * epsR[static_cast<size_t>(g) * nc + ig]));
      r[0].add(t.scaled(vcoul[igp]).scaled(0.5));
    }
    // SX of the occupied bands (:279-389)
    if (flag_occ) {
      for (int iw = 0; iw < ne; ++iw) {
        const double wx = freqevalmin - ekq[n1] + iw * freqevalstep;
        const bool pos = wx >= 0.0;
        const int f = ff_interval(pos ? wx : -wx, dFreqGrid, nfreq);
        const double d = dFreqGrid[f + 1] - dFreqGrid[f];
        const double f1 = pos ? (dFreqGrid[f + 1] - wx) / d : (dFreqGrid[f + 1] + wx) / d;
        const double f2 = pos ? (wx - dFreqGrid[f]) / d : (-dFreqGrid[f] - wx) / d;
        const cd* src = pos ? epsR : epsA;
        const cd v = ff_weighted_pair(n1, ncouls, ngpown, igp_of, aqsm, aqsn, vcoul, src + f * slab,
                                      nullptr, src + (f + 1) * slab, nullptr, f1, f2, 1.0);
        asx[iw].add(v * occ);
      }
    }
    // CH from schDt (:459-521)
    for (int f = 0; f < nfreq; ++f) {
      const cd sd = sdt[static_cast<size_t>(n1) * nfreq + f];
      const double zb = dFreqGrid[f];
      const cd coh = cd(zb, 0.0) - brd[f];
      const cd cor = flag_occ ? -1.0 * cd(zb, 0.0) - brd[f] : cd(zb, 0.0) - brd[f];
      cd left(0.0), lin(0.0), lin2(0.0), avg(0.0);
      double zr = 0.0, zl = 0.0;
      if (f != 0) {
        zr = zb;
        zl = dFreqGrid[f - 1];
        const cd right = sd;
        left = sdt[static_cast<size_t>(n1) * nfreq + f - 1];
        avg = 0.5 * (right + left);
        lin = right - left;
        lin2 = lin / (zr - zl);
      }
      if (f != nfreq - 1)
        for (int iw = 0; iw < ne; ++iw) {
          const double wx = freqevalmin - ekq[n1] + iw * freqevalstep;
          schDi[iw].add(-(cd(0.0, pref[f]) * sd / (wx - coh)));
          schDi_corb[iw].add(-(cd(0.0, pref[f]) * sd / (wx - cor)));
        }
      if (f != 0)
        for (int iw = 0; iw < ne; ++iw) {
          const double e = freqevalmin - ekq[n1] + iw * freqevalstep;
          double t = std::fabs((e - zr) / (e - zl));
          if (t < 1e-4) t = 1e-4;
          if (t > 1e4) t = 1e4;
          t = -std::log(t);
          sch2Di[iw].add(-(cd(0.0, pref_zb) * avg * t));
          cd lin3;
          if (flag_occ) {
            double t4 = std::fabs((e + zr) / (e + zl));
            if (t4 < 1e-4) t4 = 1e-4;
            if (t4 > 1e4) t4 = 1e4;
            t4 = std::log(t4);
            lin3 = (left + lin2 * (-freqevalmin - ekq[n1] + iw * freqevalstep - zl)) * t4;
          } else {
            lin3 = (left + lin2 * (e - zl)) * t;
          }
          lin3 = lin3 + lin;
          schDi_cor[iw].add(-(cd(0.0, pref_zb) * lin3));
        }
    }
    // delta-function contributions (:530-613)
    for (int iw = 0; iw < ne; ++iw) {
      const double wx = freqevalmin - ekq[n1] + iw * freqevalstep;
      if (wx >= 0.0) {
        const int f = ff_interval(wx, dFreqGrid, nfreq);
        const double d = dFreqGrid[f + 1] - dFreqGrid[f];
        const double f1 = -0.5 * (dFreqGrid[f + 1] - wx) / d;
        const double f2 = -0.5 * (wx - dFreqGrid[f]) / d;
        const cd v = ff_weighted_pair(n1, ncouls, ngpown, igp_of, aqsm, aqsn, vcoul, epsR + f * slab,
                                      epsA + f * slab, epsR + (f + 1) * slab, epsA + (f + 1) * slab, f1,
                                      f2, 1.0);
        sch2Di[iw].add(v);
        if (!flag_occ) schDi_cor[iw].add(v);
      } else if (flag_occ) {
        const double w = -wx;
        const int f = ff_interval(w, dFreqGrid, nfreq);
        const double d = dFreqGrid[f + 1] - dFreqGrid[f];
        const double f1 = (dFreqGrid[f + 1] - w) / d;
        const double f2 = (w - dFreqGrid[f]) / d;
        const cd v = ff_weighted_pair(n1, ncouls, ngpown, igp_of, aqsm, aqsn, vcoul, epsR + f * slab,
                                      epsA + f * slab, epsR + (f + 1) * slab, epsA + (f + 1) * slab, f1,
                                      f2, -0.5);
        schDi_cor[iw].add(v);
      }
    }
  }
  CDD achs;
  std::vector<CDD> tot(static_cast<size_t>(5) * ne);
  for (int n1 = 0; n1 < number_bands; ++n1) {
    const CDD* r = &per[static_cast<size_t>(n1) * (1 + 5 * ne)];
    achs.add(r[0]);
    for (int k = 0; k < 5 * ne; ++k) tot[k].add(r[1 + k]);
  }
  auto put = [](double* out, const CDD& v) {
    const cd x = v.value();
    out[0] = x.real();
    out[1] = x.imag();
  };
  put(achsDtemp, achs);
  for (int iw = 0; iw < ne; ++iw) {
    put(asxDtemp + 2 * iw, tot[iw]);
    put(achDtemp + 2 * iw, tot[ne + iw]);
    put(achDtemp_cor + 2 * iw, tot[2 * ne + iw]);
    put(achDtemp_corb + 2 * iw, tot[3 * ne + iw]);
    put(ach2Dtemp + 2 * iw, tot[4 * ne + iw]);
  }
  return kOk;
}

// ---------------------------------------------------------------------------
// Real-valued GPP (gppKer_real.cpp:17-155, 302-390): the same loop nest with
// real arrays, mygpvar1 = aqsm[n1][igp] (no conjugate), the same pole guard,
// and in the occupied-band solver ssx = Omega2 / wx^2 or
// -Omega2 cden delw / cden^2 with cden = 4 wtilde^2 (delw + 1/2).  Terms in
// the reference's operation order, double-double sums.  Where the
// reference's unoccupied loop leaves scha[ig] from an earlier frequency or
// block when the guard drops a term (:367-371 writes it only when kept), the
// oracle adds 0, the value the guard means.
namespace {

inline void real_occ(double wxt, double wtilde, double ieps, double matngmatmgp, double& ssxa,
                     double& scha) {
  const double wtilde2 = wtilde * wtilde;
  const double Omega2 = wtilde2 * ieps;
  const double wdiff = wxt - wtilde;
  double cden = wdiff;
  double rden = 1 / (cden * cden);
  const double delw = wtilde * cden * rden;
  const double delwr = delw * delw;
  const double wdiffr = wdiff * wdiff;
  double sch, ssx;
  if ((wdiffr > kLimitTwo) && (delwr < kLimitOne)) {
    sch = delw * ieps;
    cden = wxt * wxt;
    rden = cden * cden;
    rden = 1.00 / rden;
    ssx = Omega2 * cden * rden;
  } else if (delwr > kTo1) {
    sch = 0.0;
    cden = 4.00 * wtilde2 * (delw + 0.50);
    rden = cden * cden;
    rden = 1.00 / rden;
    ssx = -Omega2 * cden * rden * delw;
  } else {
    sch = 0.0;
    ssx = 0.0;
  }
  ssxa = matngmatmgp * ssx;
  scha = matngmatmgp * sch;
}

}  // namespace

extern "C" int oracle_gpp_real(int number_bands, int nvband, int ncouls, int ngpown,
                               const int* inv_igp_index, const int* indinv, int indinv_len,
                               const double* wx, double occ, const double* aqsm,
                               const double* aqsn, const double* ieps, const double* wt,
                               const double* vcoul, double* achtemp, double* asxtemp,
                               double* acht_n1_loc, int nthreads) {
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0 || nvband < 0 || nvband > number_bands)
    return kErrShape;
  std::vector<int> igp_of(ngpown);
  for (int g = 0; g < ngpown; ++g) {
    const int v = map_igp(inv_igp_index, indinv, indinv_len, ncouls, g);
    if (v == -2) return kErrIndex;
    igp_of[g] = v;
  }
  const size_t nc = static_cast<size_t>(ncouls);
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  // per band: ach[3], asx[3]
  std::vector<DD> per(static_cast<size_t>(number_bands) * 6);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int n1 = 0; n1 < number_bands; ++n1) {
    DD* r = &per[static_cast<size_t>(n1) * 6];
    const bool flag_occ = n1 < nvband;
    for (int g = 0; g < ngpown; ++g) {
      const int igp = igp_of[g];
      if (igp < 0) continue;
      const double mygpvar1 = aqsm[n1 * nc + igp];
      for (int iw = 0; iw < 3; ++iw) {
        const double wxt = wx[iw];
        DD scht, ssxt;
        for (size_t ig = 0; ig < nc; ++ig) {
          const double w = wt[g * nc + ig], e = ieps[g * nc + ig];
          if (flag_occ) {
            double ssxa, scha;
            real_occ(wxt, w, e, aqsn[n1 * nc + ig] * mygpvar1, ssxa, scha);
            dd_add(ssxt, ssxa);
            dd_add(scht, scha);
          } else {
            const double wdiff = wxt - w;
            double cden = wdiff;
            double rden = cden * cden;
            rden = 1 / rden;
            const double delw = w * cden * rden;
            const double delwr = delw * delw;
            const double wdiffr = wdiff * wdiff;
            if ((wdiffr > kLimitTwo) && (delwr < kLimitOne))
              dd_add(scht, mygpvar1 * aqsn[n1 * nc + ig] * delw * e);
          }
        }
        dd_add(r[iw], dd_mul(dd_mul(scht, 0.5), vcoul[igp]));
        if (flag_occ) dd_add(r[3 + iw], dd_mul(dd_mul(ssxt, occ), vcoul[igp]));
      }
    }
  }
  DD ach[3], asx[3];
  for (int n1 = 0; n1 < number_bands; ++n1) {
    for (int k = 0; k < 3; ++k) {
      dd_add(ach[k], per[static_cast<size_t>(n1) * 6 + k]);
      dd_add(asx[k], per[static_cast<size_t>(n1) * 6 + 3 + k]);
    }
    if (acht_n1_loc) acht_n1_loc[n1] = per[static_cast<size_t>(n1) * 6 + 2].hi + per[static_cast<size_t>(n1) * 6 + 2].lo;
  }
  for (int k = 0; k < 3; ++k) {
    achtemp[k] = ach[k].hi + ach[k].lo;
    asxtemp[k] = asx[k].hi + asx[k].lo;
  }
  return kOk;
}
