// msfem_kernel3d.cuh -- 3D multiscale-basis kernels (not yet built).
#pragma once

#include "msfem_common.cuh"

namespace msfem {

inline int pick3d_kernel(int nmax, bool mixed, const void **fn, int *nt, size_t *smem) {
  (void)nmax; (void)mixed; (void)fn; (void)nt; (void)smem;
  return -1;
}

}  // namespace msfem
