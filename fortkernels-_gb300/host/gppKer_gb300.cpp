// Command-line driver with the reference's interface, running the GPP sum
// through the sigma C ABI on the GPU.
//
//   ./gppKer_gb300 <number_bands> <number_valence_bands> <number_plane_waves>
//                  <nodes_per_mpi_group> [--mixed] [--seed S]
//
// Argument handling, shapes, the constant fill, the index maps and the
// frequencies follow BGW-Kernels/gppKer.cpp:161-314; its loop nest :303-439
// is replaced by one sigma_gpp_fp64 (or sigma_gpp_mixed) call; the report
// prints achtemp with 15 digits and the wall time like :441-446.  With
// --seed the arrays get the seeded production value ranges instead of the
// constant fill (same generator as fortkernels-_gb300/workload.py).
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <vector>

#include "sigma_gpp.h"

namespace {

struct SplitMix {
  static uint64_t fmix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // draw k of stream (seed, array_id) as a double in [0, 1)
  static double u01(uint64_t seed, uint64_t array_id, uint64_t k) {
    const uint64_t s0 = fmix(seed * 0xD1342543DE82EF95ull + array_id);
    return static_cast<double>(fmix(s0 + (k + 1) * 0x9E3779B97F4A7C15ull) >> 11) * 0x1.0p-53;
  }
};

void fill_complex(std::vector<std::complex<double>>& a, uint64_t seed, uint64_t id, double rlo,
                  double rhi, double ilo, double ihi) {
  for (size_t k = 0; k < a.size(); ++k)
    a[k] = {rlo + (rhi - rlo) * SplitMix::u01(seed, id, 2 * k),
            ilo + (ihi - ilo) * SplitMix::u01(seed, id, 2 * k + 1)};
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) {
    std::cout << "The correct form of input is : " << std::endl;
    std::cout << " ./gppKer_gb300 <number_bands> <number_valence_bands> <number_plane_waves> "
                 "<nodes_per_mpi_group> [--mixed] [--seed S]"
              << std::endl;
    return 1;
  }
  const int number_bands = std::atoi(argv[1]);
  const int nvband = std::atoi(argv[2]);
  const int ncouls = std::atoi(argv[3]);
  const int nodes_per_group = std::atoi(argv[4]);
  bool mixed = false;
  long long seed = -1;
  for (int i = 5; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--mixed")) mixed = true;
    if (!std::strcmp(argv[i], "--seed") && i + 1 < argc) seed = std::atoll(argv[++i]);
  }
  if (nodes_per_group <= 0 || ncouls <= 0) {
    std::cout << "invalid arguments" << std::endl;
    return 1;
  }
  const int npes = 1;
  const int ngpown = ncouls / (nodes_per_group * npes);
  const double e_lk = 10, dw = 1, to1 = 1e-6, e_n1kq = 6.0;
  const int nstart = 0, nend = 3;

  std::cout << "number_bands = " << number_bands << "\t nvband = " << nvband
            << "\t ncouls = " << ncouls << "\t nodes_per_group  = " << nodes_per_group
            << "\t ngpown = " << ngpown << "\t precision = " << (mixed ? "mixed" : "fp64")
            << std::endl;

  using cd = std::complex<double>;
  std::vector<cd> aqsm((size_t)number_bands * ncouls, cd(0.5, 0.5));
  std::vector<cd> aqsn((size_t)number_bands * ncouls, cd(0.5, 0.5));
  std::vector<cd> ieps((size_t)ngpown * ncouls, cd(0.5, 0.5));
  std::vector<cd> wtilde((size_t)ngpown * ncouls, cd(0.5, 0.5));
  std::vector<double> vcoul(ncouls, 1.0);
  if (seed >= 0) {
    fill_complex(aqsm, seed, 1, -1, 1, -1, 1);
    fill_complex(aqsn, seed, 2, -1, 1, -1, 1);
    fill_complex(ieps, seed, 3, -1, 1, -1, 1);
    fill_complex(wtilde, seed, 4, 0.5, 5.0, -0.1, 0.1);
    for (int i = 0; i < ncouls; ++i) vcoul[i] = 0.1 + 9.9 * SplitMix::u01(seed, 5, i);
  }
  std::vector<int> inv_igp_index(ngpown), indinv(ncouls);
  for (int ig = 0; ig < ngpown; ++ig) inv_igp_index[ig] = (int)((long long)(ig + 1) * ncouls / ngpown);
  for (int ig = 0; ig < ncouls; ++ig) indinv[ig] = ig;
  double wx_array[3];
  for (int iw = nstart; iw < nend; ++iw) {
    wx_array[iw] = e_lk - e_n1kq + dw * ((iw + 1) - 2);
    if (std::abs(wx_array[iw]) < to1) wx_array[iw] = to1;
  }
  cd achtemp[3], asxtemp[3];
  std::vector<cd> acht_n1_loc(number_bands);

  auto start = std::chrono::high_resolution_clock::now();
  auto fn = mixed ? sigma_gpp_mixed : sigma_gpp_fp64;
  const int st = fn(number_bands, nvband, ncouls, ngpown, nstart, nend, inv_igp_index.data(),
                    indinv.data(), wx_array, 1.0,
                    reinterpret_cast<const sigma_complex128*>(aqsm.data()),
                    reinterpret_cast<const sigma_complex128*>(aqsn.data()),
                    reinterpret_cast<const sigma_complex128*>(ieps.data()),
                    reinterpret_cast<const sigma_complex128*>(wtilde.data()), vcoul.data(),
                    reinterpret_cast<sigma_complex128*>(achtemp),
                    reinterpret_cast<sigma_complex128*>(asxtemp),
                    reinterpret_cast<sigma_complex128*>(acht_n1_loc.data()), nullptr);
  std::chrono::duration<double> elapsed = std::chrono::high_resolution_clock::now() - start;
  if (st != SIGMA_OK) {
    std::cout << "sigma_gpp failed: " << sigma_status_string(st) << " " << sigma_last_error_message()
              << std::endl;
    return 2;
  }
  for (int iw = nstart; iw < nend; ++iw)
    std::cout << "achtemp[" << iw << "] = " << std::setprecision(15) << achtemp[iw] << std::endl;
  for (int iw = nstart; iw < nend; ++iw)
    std::cout << "asxtemp[" << iw << "] = " << std::setprecision(15) << asxtemp[iw] << std::endl;
  std::cout << "********** Chrono Time Taken **********= " << elapsed.count() << " secs" << std::endl;
  sigma_shutdown();
  return 0;
}
