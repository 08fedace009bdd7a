// msfem_launch.h -- host-side interface between the C-ABI layer (msfem_gpu.cu)
// and the translation units that instantiate the kernels (k2d.cu, k3d_fp64.cu,
// k3d_mixed.cu, cnn_tc.cu), so the kernel families compile in parallel.
#pragma once

#include <cstddef>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "msfem_common.cuh"

namespace msfem {

// One compiled launch shape of the basis kernel.
struct Launch {
  const void *fn;
  int nt;
  size_t smem;
  int rows;          // nodes per thread strip (mixed kernels), 0 otherwise
  int minb;          // CTAs per SM the kernel was compiled for
  size_t slot_bytes; // per-CTA (per-cluster) global workspace (3D kernels), 0 = none
  int poly;          // degree of the inner polynomial preconditioner (mixed 2D), 0 = none
  int cluster = 1;   // CTAs per thread-block cluster sharing one cell (3D), 1 = none
  int coarse = 0;    // coarse-grid spacing of the two-level inner preconditioner (mixed 2D), 0 = none
};

// Compiled launch shapes per N class and precision; index 0 is the default.
std::vector<Launch> candidates_2d(int nmax, bool mixed);  // k2d.cu
std::vector<Launch> candidates_3d_fp64();                 // k3d_fp64.cu
std::vector<Launch> candidates_3d_mixed();                // k3d_mixed.cu

// Energy norms of basis functions against a reference basis.
cudaError_t launch_energy_2d(int grid, cudaStream_t st, const KernelParams &p, const double *basis,
                             const double *ref, double *err, double *nrm);  // k2d.cu
cudaError_t launch_energy_3d(int grid, cudaStream_t st, const KernelParams &p, const double *basis,
                             const double *ref, double *err, double *nrm);  // k3d_fp64.cu

namespace cnn {
// Where a tensor-core convolution runs and reports pipeline timeouts.
struct ConvCtx {
  cudaStream_t stream;
  int device;
  int sm_count;
  int *err;
};
// One 3x3 convolution layer on the tcgen05 tensor cores (cnn_tc.cu):
// (cin, cout, epi) one of the network's five layer kinds.  Returns an
// msfem_status code; *msg says why on failure.
int conv_tc(const ConvCtx &c, int cin, int cout, int epi, int B, const __nv_bfloat16 *X, const __nv_bfloat16 *W,
            const float *bias, const __nv_bfloat16 *mask, void *out, int cout_real, int dil, std::string *msg);
// Weight and bias gradient of one layer on the tcgen05 tensor cores (cnn_tc.cu):
// dW [cout_real][cin_real][9] and db [cout_real] (FP32) are accumulated into
// with atomics; (xc, gc) the padded channel counts of X and G.
int wgrad_tc(const ConvCtx &c, int xc, int gc, int B, const __nv_bfloat16 *X, const __nv_bfloat16 *G, int cin_real,
             int cout_real, float *dW, float *db, int dil, std::string *msg);
}  // namespace cnn

}  // namespace msfem
