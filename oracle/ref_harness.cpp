// Harness around the UNMODIFIED reference source BGW-Kernels/gppKer.cpp.
// TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles the reference file in
// place (its main() renamed by -Dmain=gppker_reference_main) and links it with
// this file into oracle/_ref/libgppref.so.  Nothing from the reference is
// copied here: the two prototypes below declare functions that the reference
// defines, so that the harness can call them on seeded inputs.
//
//   flagOCC_solver  BGW-Kernels/gppKer.cpp:130-159 (drives ssxt_scht_solver :19-65)
//   main            BGW-Kernels/gppKer.cpp:161-449

#include <complex>
#include <cstdint>
#include <cstdio>

void flagOCC_solver(double wxt, std::complex<double>* wtilde_array_tmp, int my_igp, int n1,
                    std::complex<double>* aqsmtemp_arr, std::complex<double>* aqsntemp_arr,
                    std::complex<double>* I_eps_array_tmp, std::complex<double>& ssxt,
                    std::complex<double>& scht, int igmax, int ncouls, int igp,
                    int number_bands, int ngpown);
int gppker_reference_main(int argc, char** argv);

extern "C" {

// For every (n1, my_igp, iw) with igp = igp_of[my_igp] >= 0, calls the
// reference's flagOCC_solver over all ncouls g-vectors and stores
// ssx_array[iw] = ssxt and sch_array[iw] = 0.5 * scht exactly as
// BGW-Kernels/gppKer.cpp:341-346 forms them.  Outputs are
// [number_bands][ngpown][3] complex.  The reference solver is the per-term
// arithmetic of every band; the main loop applies it to bands n1 < nvband.
int ref_flagocc_columns(int number_bands, int ncouls, int ngpown, const int* igp_of,
                        const double* wx /*[3]*/, double* aqsmtemp, double* aqsntemp,
                        double* I_eps_array, double* wtilde_array, double* out_ssx,
                        double* out_sch) {
  using cd = std::complex<double>;
  for (int n1 = 0; n1 < number_bands; ++n1)
    for (int my_igp = 0; my_igp < ngpown; ++my_igp)
      for (int iw = 0; iw < 3; ++iw) {
        const int igp = igp_of[my_igp];
        cd ssxt(0.0, 0.0), scht(0.0, 0.0);
        if (igp >= 0)
          flagOCC_solver(wx[iw], reinterpret_cast<cd*>(wtilde_array), my_igp, n1,
                         reinterpret_cast<cd*>(aqsmtemp), reinterpret_cast<cd*>(aqsntemp),
                         reinterpret_cast<cd*>(I_eps_array), ssxt, scht, ncouls, ncouls, igp,
                         number_bands, ngpown);
        const int64_t o = (static_cast<int64_t>(n1) * ngpown + my_igp) * 3 + iw;
        cd sch = 0.5 * scht;
        out_ssx[2 * o] = ssxt.real();
        out_ssx[2 * o + 1] = ssxt.imag();
        out_sch[2 * o] = sch.real();
        out_sch[2 * o + 1] = sch.imag();
      }
  return 0;
}

// Runs the reference's own driver with argv = {prog, nb, nvband, ncouls, npg}.
// It prints its usual report (achtemp at 15 digits, chrono time) to stdout.
int ref_main(int number_bands, int nvband, int ncouls, int nodes_per_group) {
  static char prog[] = "gppKer";
  char a1[32], a2[32], a3[32], a4[32];
  snprintf(a1, sizeof a1, "%d", number_bands);
  snprintf(a2, sizeof a2, "%d", nvband);
  snprintf(a3, sizeof a3, "%d", ncouls);
  snprintf(a4, sizeof a4, "%d", nodes_per_group);
  char* argv[] = {prog, a1, a2, a3, a4, nullptr};
  return gppker_reference_main(5, argv);
}

}  // extern "C"
