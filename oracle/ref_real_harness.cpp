// Harness around the UNMODIFIED reference source gppKer_real.cpp (the
// real-valued GPP mini-app).  TEST INFRASTRUCTURE ONLY.  oracle/build.py
// compiles the reference file in place (main() renamed by
// -Dmain=gppreal_reference_main) and links it with this file into
// oracle/_ref/libgpprealref.so.  The prototype below declares the
// reference's occupied-band solver (gppKer_real.cpp:124-155) so that the
// harness can call it on seeded inputs; nothing is copied.

#include <cstdint>

void flagOCC_solver(double wxt, double* wtilde_array_tmp, int my_igp, int n1, double* aqsmtemp_arr,
                    double* aqsntemp_arr, double* I_eps_array_tmp, double& ssxt, double& scht,
                    int ncouls, int igp, int number_bands, int ngpown);

extern "C" {

// ssx_array[iw] = ssxt and sch_array[iw] = 0.5 * scht of every (n1, my_igp,
// iw) with igp = igp_of[my_igp] >= 0, as gppKer_real.cpp:331-339 forms them.
// Outputs [number_bands][ngpown][3] doubles.
int ref_real_flagocc_columns(int number_bands, int ncouls, int ngpown, const int* igp_of,
                             const double* wx, double* aqsm, double* aqsn, double* ieps, double* wt,
                             double* out_ssx, double* out_sch) {
  for (int n1 = 0; n1 < number_bands; ++n1)
    for (int g = 0; g < ngpown; ++g)
      for (int iw = 0; iw < 3; ++iw) {
        double ssxt = 0.0, scht = 0.0;
        if (igp_of[g] >= 0)
          flagOCC_solver(wx[iw], wt, g, n1, aqsm, aqsn, ieps, ssxt, scht, ncouls, igp_of[g],
                         number_bands, ngpown);
        const int64_t o = (static_cast<int64_t>(n1) * ngpown + g) * 3 + iw;
        out_ssx[o] = ssxt;
        out_sch[o] = 0.5 * scht;
      }
  return 0;
}

}  // extern "C"
