// Harness around the UNMODIFIED reference source FFKer_cori/ffKernel.cpp.
// TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles the reference file in
// place (its main() renamed by -Dmain=ffker_reference_main, its own
// Complex.h found through -I) and links it with this file into
// oracle/_ref/libffref.so.  Nothing from the reference is copied: the
// prototypes below declare functions the reference defines, and its complex
// class is only named (its layout is two doubles, re then im).
//
//   achsDtemp_Kernel     FFKer_cori/ffKernel.cpp:107-131
//   asxDtemp_Kernel      FFKer_cori/ffKernel.cpp:133-153
//   achDtemp_cor_Kernel  FFKer_cori/ffKernel.cpp:212-245

#include <vector>

class GPUComplex;

void achsDtemp_Kernel(int number_bands, int ngpown, int ncouls, int* inv_igp_index, int* indinv,
                      GPUComplex* aqsntemp, GPUComplex* aqsmtemp, GPUComplex* I_epsR_array,
                      double* vcoul, GPUComplex& achsDtemp);
void asxDtemp_Kernel(int nvband, int nfreqeval, int ncouls, int ngpown, int numThreads, int nFreq,
                     double freqevalmin, double freqevalstep, double occ, double* ekq,
                     double* dFreqGrid, int* inv_igp_index, int* indinv, GPUComplex* aqsmtemp,
                     GPUComplex* aqsntemp, double* vcoul, GPUComplex* I_epsR_array,
                     GPUComplex* ssxDittt, GPUComplex* asxDtemp);
void achDtemp_cor_Kernel(int number_bands, int nvband, int nfreqeval, int ncouls, int ngpown,
                         int nFreq, double freqevalmin, double freqevalstep, double* ekq,
                         double* dFreqGrid, int* inv_igp_index, int* indinv,
                         GPUComplex* aqsmtemp, GPUComplex* aqsntemp, double* vcoul,
                         GPUComplex* I_epsR_array, GPUComplex* I_epsA_array,
                         GPUComplex* schDi_cor, GPUComplex* schDi_corb, GPUComplex* sch2Di,
                         GPUComplex* ach2Dtemp, GPUComplex* achDtemp_cor,
                         GPUComplex* achDtemp_corb);

namespace {
GPUComplex* C(double* p) { return reinterpret_cast<GPUComplex*>(p); }
}  // namespace

extern "C" {

// The three reference kernels on caller-supplied arrays (interleaved complex
// doubles).  Outputs must be zeroed by the caller (the reference accumulates
// into asxDtemp / achDtemp_cor).  out_achs: complex[1]; out_asx and out_cor:
// complex[nfreqeval].
int ref_ff_kernels(int number_bands, int nvband, int ncouls, int ngpown, int nfreq, int nfreqeval,
                   double freqevalmin, double freqevalstep, double occ, int* inv_igp_index,
                   int* indinv, double* aqsm, double* aqsn, double* I_epsR, double* I_epsA,
                   double* vcoul, double* ekq, double* dFreqGrid, double* out_achs,
                   double* out_asx, double* out_cor) {
  std::vector<double> ssx(2 * 64, 0.0), cor(2 * nfreqeval, 0.0), corb(2 * nfreqeval, 0.0),
      sch2(2 * nfreqeval, 0.0), ach2(2 * nfreqeval, 0.0), corb_t(2 * nfreqeval, 0.0);
  achsDtemp_Kernel(number_bands, ngpown, ncouls, inv_igp_index, indinv, C(aqsn), C(aqsm), C(I_epsR),
                   vcoul, *C(out_achs));
  asxDtemp_Kernel(nvband, nfreqeval, ncouls, ngpown, 64, nfreq, freqevalmin, freqevalstep, occ, ekq,
                  dFreqGrid, inv_igp_index, indinv, C(aqsm), C(aqsn), vcoul, C(I_epsR),
                  C(ssx.data()), C(out_asx));
  achDtemp_cor_Kernel(number_bands, nvband, nfreqeval, ncouls, ngpown, nfreq, freqevalmin,
                      freqevalstep, ekq, dFreqGrid, inv_igp_index, indinv, C(aqsm), C(aqsn), vcoul,
                      C(I_epsR), C(I_epsA), C(cor.data()), C(corb.data()), C(sch2.data()),
                      C(ach2.data()), C(out_cor), C(corb_t.data()));
  return 0;
}

}  // extern "C"
