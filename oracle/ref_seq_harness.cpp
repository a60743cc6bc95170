// Harness around the UNMODIFIED reference source gppKerSeq.cpp, the
// sequential GPP driver that carries the gppsum = 1 ("half sum") variant.
// TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles the reference file in
// place (its main() renamed by -Dmain=gppseq_reference_main) and links it
// with this file into oracle/_ref/libgppseqref.so.  Nothing from the
// reference is copied: the prototypes below declare functions the reference
// defines, so that the harness can call them on seeded inputs.
//
//   reduce_achstemp   gppKerSeq.cpp:13-72
//   flagOCC_solver    gppKerSeq.cpp:76-191
//   noflagOCC_solver  gppKerSeq.cpp:193-261
//   main              gppKerSeq.cpp:263-505
//
// The reference stores its arrays g-vector-major behind row pointers
// (aqsmtemp[ig][n1], I_eps_array[ig][my_igp]); the harness takes the
// library's band-major arrays, transposes them and builds the row pointers.
// The band loop around the solvers (512-wide g-vector blocks for the
// non-occupied bands, gppKerSeq.cpp:457-470) lives in the reference's main
// and is driven here the same way.

#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <vector>

using cd = std::complex<double>;

void reduce_achstemp(int n1, int* inv_igp_index, int ncouls, cd** aqsmtemp, cd** aqsntemp,
                     cd** I_eps_array, cd& achstemp, int* indinv, int ngpown, int gppsum,
                     double* vcoul);
void flagOCC_solver(double wxt, cd** wtilde_array, int my_igp, int n1, cd** aqsmtemp,
                    cd** aqsntemp, cd** I_eps_array, int gppsum, cd& ssxt, cd& scht, int igmax,
                    int ncouls, int igp);
void noflagOCC_solver(int igbeg, int igend, int igblk, double wxt, cd** wtilde_array, int my_igp,
                      int n1, cd** aqsmtemp, cd** aqsntemp, cd** I_eps_array, int gppsum,
                      cd& ssxt, cd& scht, int igmax, int ncouls, int igp);
int gppseq_reference_main(int argc, char** argv);

namespace {

// [rows][cols] band-major complex -> [cols][rows] storage plus row pointers
struct GvecMajor {
  std::vector<cd> data;
  std::vector<cd*> rows;
  GvecMajor(const double* src, int nrows, int ncols) : data((size_t)nrows * ncols), rows(ncols) {
    const cd* s = reinterpret_cast<const cd*>(src);
    for (int r = 0; r < nrows; ++r)
      for (int c = 0; c < ncols; ++c) data[(size_t)c * nrows + r] = s[(size_t)r * ncols + c];
    for (int c = 0; c < ncols; ++c) rows[c] = data.data() + (size_t)c * nrows;
  }
};

}  // namespace

extern "C" {

// For every (n1, my_igp, iw) with igp = igp_of[my_igp] >= 0: sch_array[iw]
// and ssx_array[iw] as gppKerSeq.cpp:432-470 forms them with gppsum = 1
// (the occupied solver for n1 < nvband, the blocked non-occupied solver
// otherwise).  Outputs [nb][ng][3] complex.
int ref_seq_columns(int number_bands, int nvband, int ncouls, int ngpown, const int* igp_of,
                    const double* wx, const double* aqsmtemp, const double* aqsntemp,
                    const double* I_eps_array, const double* wtilde_array, double* out_sch,
                    double* out_ssx) {
  GvecMajor m(aqsmtemp, number_bands, ncouls), n(aqsntemp, number_bands, ncouls);
  GvecMajor e(I_eps_array, ngpown, ncouls), w(wtilde_array, ngpown, ncouls);
  const int gppsum = 1, igblk = 512;
  for (int n1 = 0; n1 < number_bands; ++n1)
    for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
      const int igp = igp_of[my_igp];
      cd ssx_array[3], sch_array[3];
      if (igp >= 0) {
        const int igmax = igp;
        if (n1 < nvband) {
          for (int iw = 0; iw < 3; ++iw) {
            cd scht(0.0, 0.0), ssxt(0.0, 0.0);
            flagOCC_solver(wx[iw], w.rows.data(), my_igp, n1, m.rows.data(), n.rows.data(),
                           e.rows.data(), gppsum, ssxt, scht, igmax, ncouls, igp);
            ssx_array[iw] += ssxt;
            sch_array[iw] += 0.5 * scht;
          }
        } else {
          for (int igbeg = 0; igbeg < igmax; igbeg += igblk) {
            const int igend = std::min(igbeg + igblk - 1, igmax);
            for (int iw = 0; iw < 3; ++iw) {
              cd scht(0.0, 0.0), ssxt(0.0, 0.0);
              noflagOCC_solver(igbeg, igend, igblk, wx[iw], w.rows.data(), my_igp, n1,
                               m.rows.data(), n.rows.data(), e.rows.data(), gppsum, ssxt, scht,
                               igmax, ncouls, igp);
              sch_array[iw] += 0.5 * scht;
            }
          }
        }
      }
      for (int iw = 0; iw < 3; ++iw) {
        const int64_t o = ((int64_t)n1 * ngpown + my_igp) * 3 + iw;
        out_sch[2 * o] = sch_array[iw].real();
        out_sch[2 * o + 1] = sch_array[iw].imag();
        out_ssx[2 * o] = ssx_array[iw].real();
        out_ssx[2 * o + 1] = ssx_array[iw].imag();
      }
    }
  return 0;
}

// achstemp after the reference's reduce_achstemp with gppsum = 1 has run for
// every band n1 = 0 .. number_bands-1 (it accumulates over the band loop,
// gppKerSeq.cpp:412).  inv_igp_index / indinv are passed through unchanged.
int ref_seq_achstemp(int number_bands, int ncouls, int ngpown, int* inv_igp_index, int* indinv,
                     const double* aqsmtemp, const double* aqsntemp, const double* I_eps_array,
                     double* vcoul, double* out) {
  GvecMajor m(aqsmtemp, number_bands, ncouls), n(aqsntemp, number_bands, ncouls);
  GvecMajor e(I_eps_array, ngpown, ncouls);
  cd achstemp(0.0, 0.0);
  for (int n1 = 0; n1 < number_bands; ++n1)
    reduce_achstemp(n1, inv_igp_index, ncouls, m.rows.data(), n.rows.data(), e.rows.data(),
                    achstemp, indinv, ngpown, 1, vcoul);
  out[0] = achstemp.real();
  out[1] = achstemp.imag();
  return 0;
}

// Runs the reference's own driver with argv = {prog, nb, nvband, ncouls, npg, gppsum}.
int ref_seq_main(int number_bands, int nvband, int ncouls, int nodes_per_group, int gppsum) {
  static char prog[] = "gppKerSeq";
  char a1[32], a2[32], a3[32], a4[32], a5[32];
  snprintf(a1, sizeof a1, "%d", number_bands);
  snprintf(a2, sizeof a2, "%d", nvband);
  snprintf(a3, sizeof a3, "%d", ncouls);
  snprintf(a4, sizeof a4, "%d", nodes_per_group);
  snprintf(a5, sizeof a5, "%d", gppsum);
  char* argv[] = {prog, a1, a2, a3, a4, a5, nullptr};
  return gppseq_reference_main(6, argv);
}

}  // extern "C"
