// k3d_mixed.cu -- the 3D basis kernel's mixed-precision launch shapes (FP32
// inner CG with FP64 refinement): one CTA per cell with register caps for
// 1-3 CTAs per SM, and thread-block clusters of 8 CTAs per cell whose inner
// CG keeps the cell's slabs in shared memory.
#include "msfem_kernel3d.cuh"
#include "msfem_launch.h"

namespace msfem {

std::vector<Launch> candidates_3d_mixed() {
  const size_t slot = Work3D::bytes(true);
  auto l3 = [&](const void *fn, int nt, int minb, int cl) {
    Launch L{fn, nt, 0, 0, minb, slot, 0};
    L.cluster = cl;
    return L;
  };
  // cluster shape: 8 CTAs of 544 threads (one per interior column of the
  // largest cell), the slabs of the inner CG in dynamic shared memory
  Launch slab = l3((const void *)msfem3d_kernel<544, true, 1, 8>, 544, 1, 8);
  slab.smem = Slab3D<(kNMax3D - 1 + 7) / 8>::bytes;
  return {l3((const void *)msfem3d_kernel<256, true, 1, 1>, 256, 1, 1),
          l3((const void *)msfem3d_kernel<512, true, 1, 1>, 512, 1, 1),
          l3((const void *)msfem3d_kernel<256, true, 2, 1>, 256, 2, 1),
          l3((const void *)msfem3d_kernel<256, true, 3, 1>, 256, 3, 1),
          l3((const void *)msfem3d_kernel<512, true, 2, 1>, 512, 2, 1),
          slab};
}

}  // namespace msfem
