// k2d.cu -- the 2D basis kernels' launch shapes (FP64 form, mixed forms,
// energy norms), compiled apart from the C-ABI layer.
#include "msfem_kernel2d.cuh"
#include "msfem_launch.h"

namespace msfem {
namespace {

template <int NMAX, int NT>
Launch make2d() {
  return Launch{(const void *)msfem2d_kernel<NMAX, NT>, NT, Smem2D<NMAX>::bytes(false), 0, 2, 0, 0};
}
template <int NMAX, int NT, int S, int MINB, int M = 0, int CH = 0>
Launch make2d_mixed() {
  using L = Smem2D<NMAX>;
  // the polynomial-preconditioned form needs a second exchange buffer unless
  // it runs two CTAs per SM (one buffer, one more barrier per Chebyshev step);
  // the two-level form adds its coarse-grid arrays
  const size_t smem = CH > 0 ? Coarse2D<NMAX, CH>::kEnd : (M > 0 && MINB < 2) ? L::kEndCheb : L::bytes(true);
  return Launch{(const void *)msfem2d_mixed_kernel<NMAX, NT, S, MINB, M, CH>, NT, smem, S, MINB, 0,
                M > 0 ? M - 1 : 0, 1, CH};
}

}  // namespace

std::vector<Launch> candidates_2d(int nmax, bool mixed) {
  if (nmax <= 16) {
    if (mixed)
      return {make2d_mixed<16, 128, 2, 2>(), make2d_mixed<16, 64, 4, 4>(), make2d_mixed<16, 128, 2, 1>(),
              make2d_mixed<16, 128, 2, 1, 4>()};
    return {make2d<16, 128>()};
  }
  if (mixed)
    return {make2d_mixed<32, 256, 4, 2>(), make2d_mixed<32, 256, 4, 1>(), make2d_mixed<32, 512, 2, 1>(),
            // polynomial-preconditioned inner CG (degree M - 1 Chebyshev)
            make2d_mixed<32, 512, 2, 1, 4>(), make2d_mixed<32, 512, 2, 1, 6>(), make2d_mixed<32, 256, 4, 1, 4>(),
            make2d_mixed<32, 256, 4, 1, 6>(), make2d_mixed<32, 256, 4, 2, 4>(), make2d_mixed<32, 256, 4, 2, 6>(),
            // two-level V-cycle: Chebyshev smoothing of degree M - 1 = 2 around a
            // Galerkin coarse-grid correction of spacing 4 (degree 3 measured
            // 1-3 % slower on the 64x64- and 256x256-cell fields)
            make2d_mixed<32, 256, 4, 1, 3, 4>()};
  return {make2d<32, 256>()};
}

cudaError_t launch_energy_2d(int grid, cudaStream_t st, const KernelParams &p, const double *basis,
                             const double *ref, double *err, double *nrm) {
  msfem2d_energy_kernel<256><<<grid, 256, 0, st>>>(p, basis, ref, err, nrm);
  return cudaGetLastError();
}

}  // namespace msfem
