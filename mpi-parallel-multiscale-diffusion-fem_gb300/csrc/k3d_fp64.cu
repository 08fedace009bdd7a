// k3d_fp64.cu -- the 3D basis kernel's FP64 launch shapes (one CTA per cell
// with register caps for 1-3 CTAs per SM, and thread-block clusters of 8
// CTAs per cell) and the 3D energy-norm kernel.
#include "msfem_kernel3d.cuh"
#include "msfem_launch.h"

namespace msfem {

std::vector<Launch> candidates_3d_fp64() {
  const size_t slot = Work3D::bytes(false);
  auto l3 = [&](const void *fn, int nt, int minb, int cl) {
    Launch L{fn, nt, 0, 0, minb, slot, 0};
    L.cluster = cl;
    return L;
  };
  return {l3((const void *)msfem3d_kernel<256, false, 1, 1>, 256, 1, 1),
          l3((const void *)msfem3d_kernel<512, false, 1, 1>, 512, 1, 1),
          l3((const void *)msfem3d_kernel<256, false, 2, 1>, 256, 2, 1),
          l3((const void *)msfem3d_kernel<256, false, 3, 1>, 256, 3, 1),
          l3((const void *)msfem3d_kernel<512, false, 2, 1>, 512, 2, 1),
          l3((const void *)msfem3d_kernel<512, false, 1, 8>, 512, 1, 8)};
}

cudaError_t launch_energy_3d(int grid, cudaStream_t st, const KernelParams &p, const double *basis,
                             const double *ref, double *err, double *nrm) {
  msfem3d_energy_kernel<256><<<grid, 256, 0, st>>>(p, basis, ref, err, nrm);
  return cudaGetLastError();
}

}  // namespace msfem
