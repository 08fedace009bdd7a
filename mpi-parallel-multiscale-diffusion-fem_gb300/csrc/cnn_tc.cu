// cnn_tc.cu -- host side of the warm-start network's tcgen05 convolution:
// TMA tensor maps (cuTensorMapEncodeTiled from the driver), launch geometry,
// and the five instantiated layer kinds.
#include <algorithm>
#include <mutex>
#include <string>

#include <cuda.h>

#include "msfem_cnn.cuh"
#include "msfem_conv_tc.cuh"
#include "msfem_gpu.h"
#include "msfem_launch.h"

namespace msfem {
namespace cnn {
namespace {

using bf16 = __nv_bfloat16;

int fail(std::string *msg, int code, const std::string &m) {
  if (msg) *msg = m;
  return code;
}
#define CONV_CUDA(call)                                                            \
  do {                                                                             \
    const cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) return fail(msg, MSFEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn tensor_map_encoder() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// One 3x3 convolution layer on the tcgen05 tensor cores: X (channel-blocked
// bf16) through a TMA tensor map (one box of (33 + 2 dil) pixels x the window
// rows per 8-channel block), persistent CTAs capped so that their TMEM
// columns fit the SM's 512.
template <int CIN, int COUT, int EPI>
int conv_tc_t(const ConvCtx &c, int B, const bf16 *X, const bf16 *W, const float *bias, const bf16 *mask,
              void *out, int cout_real, int dil, std::string *msg) {
  if (B <= 0) return MSFEM_OK;
  const EncodeTiledFn enc = tensor_map_encoder();
  if (!enc) return fail(msg, MSFEM_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const tc::ConvGeom g = tc::conv_geom(dil);
  // blocked layout [B][CIN/8][33][33][8] viewed as 8-byte elements: dims (66
  // per row = 33 pixels x 2, 33 rows, B * CIN/8 blocks); a box row is a
  // contiguous run of wp pixels (2 wp elements <= 98, within the 256 limit).
  // Two maps: boxes of kBoxRows rows and one of the remaining window rows.
  const cuuint64_t dims[3] = {2u * kW, (cuuint64_t)kH, (cuuint64_t)B * (CIN / 8)};
  const cuuint64_t strides[2] = {(cuuint64_t)kW * 16, (cuuint64_t)kPix * 16};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  const int rem = g.box_rows % tc::kBoxRows;
  CUtensorMap maps[2];
  for (int m = 0; m < 2; ++m) {
    const cuuint32_t rows = m == 0 ? (cuuint32_t)tc::kBoxRows : (cuuint32_t)std::max(rem, 1);
    const cuuint32_t box[3] = {2u * (cuuint32_t)g.wp, rows, 1u};
    const CUresult r = enc(&maps[m], CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<bf16 *>(X), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
      return fail(msg, MSFEM_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  }
  auto fn = tc::conv3x3_tc_kernel<CIN, COUT, EPI>;
  const size_t smem = tc::conv_tc_smem<CIN, COUT>(dil);
  CONV_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)tc::conv_tc_smem<CIN, COUT>(kMaxDil)));
  // all of the unified L1/shared storage as shared memory, so that several
  // CTAs fit from the first launch on
  CONV_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
  // CTAs per SM from the shared-memory capacity and the 512 TMEM columns
  // (an SM never holds more accumulator sets than fit)
  int smem_sm = 0, smem_rsv = 0;
  CONV_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c.device));
  CONV_CUDA(cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, c.device));
  int per_sm = smem_sm / (int)(smem + smem_rsv + 256);  // + static shared memory (<= 208 B)
  per_sm = std::min(per_sm, 512 / (tc::kStages * tc::kTiles * COUT));
  if (per_sm < 1) return fail(msg, MSFEM_ERR_UNSUPPORTED, "tensor-core convolution does not fit on an SM");
  const long items = (long)B * g.segs;
  const int grid = (int)std::min<long>(items, (long)per_sm * c.sm_count);
  fn<<<grid, tc::kThreads, smem, c.stream>>>(maps[0], maps[1], W, bias, mask, out, cout_real, dil, B,
                                                      c.err);
  CONV_CUDA(cudaGetLastError());
  return MSFEM_OK;
}

// Weight and bias gradient of one layer on the tcgen05 tensor cores: X
// through the same kind of tensor map as the forward pass (the window rows of
// 256-position items), G read directly.
template <int XC, int GC>
int wgrad_tc_t(const ConvCtx &c, int B, const bf16 *X, const bf16 *G, int cin_real, int cout_real, float *dW,
               float *db, int dil, std::string *msg) {
  if (B <= 0) return MSFEM_OK;
  const EncodeTiledFn enc = tensor_map_encoder();
  if (!enc) return fail(msg, MSFEM_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const tc::WgGeom g = tc::wg_geom(dil);
  const cuuint64_t dims[3] = {2u * kW, (cuuint64_t)kH, (cuuint64_t)B * (XC / 8)};
  const cuuint64_t strides[2] = {(cuuint64_t)kW * 16, (cuuint64_t)kPix * 16};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  const int rem = g.box_rows % tc::kBoxRows;
  CUtensorMap maps[2];
  for (int m = 0; m < 2; ++m) {
    const cuuint32_t rows = m == 0 ? (cuuint32_t)tc::kBoxRows : (cuuint32_t)std::max(rem, 1);
    const cuuint32_t box[3] = {2u * (cuuint32_t)g.wp, rows, 1u};
    const CUresult r = enc(&maps[m], CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<bf16 *>(X), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
      return fail(msg, MSFEM_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  }
  auto fn = tc::conv3x3_wgrad_tc_kernel<XC, GC>;
  const size_t smem = tc::wgrad_tc_smem<XC>(dil);
  CONV_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)tc::wgrad_tc_smem<XC>(kMaxDil)));
  CONV_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
  int smem_sm = 0, smem_rsv = 0;
  CONV_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c.device));
  CONV_CUDA(cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, c.device));
  int per_sm = smem_sm / (int)(smem + smem_rsv + 256);
  per_sm = std::min(per_sm, (int)(512 / tc::wgrad_tmem_cols<XC>()));
  if (per_sm < 1) return fail(msg, MSFEM_ERR_UNSUPPORTED, "tensor-core weight gradient does not fit on an SM");
  const long items = (long)B * g.segs;
  const int grid = (int)std::min<long>(items, (long)per_sm * c.sm_count);
  fn<<<grid, tc::kWgThreads, smem, c.stream>>>(maps[0], maps[1], G, B, cin_real, cout_real, dW, db, dil, c.err);
  CONV_CUDA(cudaGetLastError());
  return MSFEM_OK;
}

}  // namespace

int wgrad_tc(const ConvCtx &c, int xc, int gc, int B, const bf16 *X, const bf16 *G, int cin_real, int cout_real,
             float *dW, float *db, int dil, std::string *msg) {
  if (xc == 32 && gc == 16) return wgrad_tc_t<32, 16>(c, B, X, G, cin_real, cout_real, dW, db, dil, msg);
  if (xc == 32 && gc == 32) return wgrad_tc_t<32, 32>(c, B, X, G, cin_real, cout_real, dW, db, dil, msg);
  if (xc == 16 && gc == 32) return wgrad_tc_t<16, 32>(c, B, X, G, cin_real, cout_real, dW, db, dil, msg);
  return fail(msg, MSFEM_ERR_UNSUPPORTED, "no compiled weight gradient for this layer kind");
}

int conv_tc(const ConvCtx &c, int cin, int cout, int epi, int B, const bf16 *X, const bf16 *W, const float *bias,
            const bf16 *mask, void *out, int cout_real, int dil, std::string *msg) {
  if (cin == 16 && cout == 32 && epi == EPI_RELU_BF16)
    return conv_tc_t<16, 32, EPI_RELU_BF16>(c, B, X, W, bias, mask, out, cout_real, dil, msg);
  if (cin == 32 && cout == 32 && epi == EPI_RELU_BF16)
    return conv_tc_t<32, 32, EPI_RELU_BF16>(c, B, X, W, bias, mask, out, cout_real, dil, msg);
  if (cin == 32 && cout == 16 && epi == EPI_F32_NCHW)
    return conv_tc_t<32, 16, EPI_F32_NCHW>(c, B, X, W, bias, mask, out, cout_real, dil, msg);
  if (cin == 16 && cout == 32 && epi == EPI_MASK_BF16)
    return conv_tc_t<16, 32, EPI_MASK_BF16>(c, B, X, W, bias, mask, out, cout_real, dil, msg);
  if (cin == 32 && cout == 32 && epi == EPI_MASK_BF16)
    return conv_tc_t<32, 32, EPI_MASK_BF16>(c, B, X, W, bias, mask, out, cout_real, dil, msg);
  return fail(msg, MSFEM_ERR_UNSUPPORTED, "no compiled convolution for this layer kind");
}

}  // namespace cnn
}  // namespace msfem
