// msfem_cnn.cuh -- the learned warm start: a 6-layer 3x3 convolutional
// network that maps the coefficient of a 2D cell (on its 33 x 33 fine nodal
// grid, N = 32) to the four multiscale basis functions, used as the initial
// guess of the local CG (which still runs to the same tolerance).  The
// reference has no counterpart; the network is trained on basis solves this
// library itself produces.
//
//   input    3 channels per node: log a11, a12 / sqrt(a11 a22), log a22
//            (the tabulated tensor averaged over the node's fine cells)
//   layers   3 -> 32 -> 32 -> 32 -> 32 -> 32 -> 4, 3x3 kernels with dilations
//            1, 2, 4, 8, 2, 1 (receptive field 37 x 37: every node sees the
//            whole cell), 'same' zero padding, ReLU after layers 1-5;
//            output = delta_i = phi_i - Q1_i at every node
//   numerics BF16 weights and activations, FP32 accumulation on the tensor
//            cores (tcgen05.mma kind::f16 with TMEM accumulators, in
//            msfem_conv_tc.cuh) for the forward pass, the input gradient
//            and the weight/bias gradient; FP32 master weights and Adam.
//
// Device layouts: activations channel-blocked BF16 [B][C/8][33][33][8] (8
// channels = 16 bytes per pixel and block; C padded to 16 or 32: first layer
// 16 channels with 3 used, last layer 16 with 4 used), so that one TMA box row
// is a contiguous run of pixels and the epilogue stores are coalesced.
// Weights for the forward pass [Cout][9][Cin], for the input-gradient pass
// (transposed, taps flipped) [Cin][9][Cout].
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace msfem {
namespace cnn {

constexpr int kH = 33, kW = 33, kPix = kH * kW;
constexpr int kLayers = 6;
// real and padded channel counts per layer boundary (0 = input)
__host__ __device__ constexpr int real_ch(int i) { return i == 0 ? 3 : (i == kLayers ? 4 : 32); }
__host__ __device__ constexpr int pad_ch(int i) { return i == 0 ? 16 : (i == kLayers ? 16 : 32); }
// dilation of layer l (0-based)
__host__ __device__ constexpr int dilation(int l) { return l == 1 ? 2 : (l == 2 ? 4 : (l == 3 ? 8 : (l == 4 ? 2 : 1))); }
constexpr int kMaxDil = 8;

// FP32 parameter vector: for each layer W [Cout][Cin][3][3] then b [Cout] (real sizes).
__host__ __device__ constexpr long param_offset(int layer) {
  long off = 0;
  for (int l = 0; l < layer; ++l) off += (long)real_ch(l + 1) * real_ch(l) * 9 + real_ch(l + 1);
  return off;
}
constexpr long kParams = param_offset(kLayers);

// Epilogue modes of the convolution kernel.
enum { EPI_RELU_BF16 = 0,   // out = bf16(relu(acc + b))          (hidden layers)
       EPI_F32_NCHW = 1,    // out = float(acc + b), NCHW, real channels (last layer)
       EPI_MASK_BF16 = 2 }; // out = bf16(acc * [mask > 0])       (input gradient)

// The weight/bias gradient runs on the tensor cores (conv3x3_wgrad_tc_kernel,
// msfem_conv_tc.cuh).

// Pack the FP32 parameters of layer l into the BF16 forward layout
// [COUTp][9][CINp] and the transposed, tap-flipped layout [CINp][9][COUTp]
// used by the input-gradient pass.
static __global__ void pack_layer_kernel(const float *__restrict__ params, int layer, __nv_bfloat16 *__restrict__ wf,
                                  __nv_bfloat16 *__restrict__ wt, float *__restrict__ bias_pad) {
  const int cin = real_ch(layer), cout = real_ch(layer + 1);
  const int cinp = pad_ch(layer), coutp = pad_ch(layer + 1);
  const float *W = params + param_offset(layer);
  const float *bb = W + (long)cout * cin * 9;
  const int total = coutp * 9 * cinp;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int co = i / (9 * cinp), tap = (i / cinp) % 9, ci = i % cinp;
    const float v = (co < cout && ci < cin) ? W[((long)co * cin + ci) * 9 + tap] : 0.f;
    wf[i] = __float2bfloat16(v);
    // transposed: row ci, tap flipped (8 - tap), column co
    wt[((long)ci * 9 + (8 - tap)) * coutp + co] = __float2bfloat16(v);
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < coutp; i += gridDim.x * blockDim.x)
    bias_pad[i] = i < cout ? bb[i] : 0.f;
}

// Features NCHW FP32 [B][3][33][33] -> channel-blocked BF16 [B][2][33][33][8]
// (16 channels, 3 used).
static __global__ void features_to_blocked_kernel(const float *__restrict__ f, int B, __nv_bfloat16 *__restrict__ x) {
  const long total = (long)B * kPix;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long b = i / kPix, p = i % kPix;
    __align__(16) __nv_bfloat16 c0[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) c0[c] = __float2bfloat16(c < 3 ? f[(b * 3 + c) * kPix + p] : 0.f);
    *reinterpret_cast<uint4 *>(x + ((b * 2 + 0) * kPix + p) * 8) = *reinterpret_cast<const uint4 *>(c0);
    *reinterpret_cast<uint4 *>(x + ((b * 2 + 1) * kPix + p) * 8) = make_uint4(0, 0, 0, 0);
  }
}

// MSE loss over interior nodes and its gradient (channel-blocked BF16
// [B][2][33][33][8], 16 channels, 4 used).
static __global__ void mse_loss_kernel(const float *__restrict__ pred, const float *__restrict__ tgt, int B,
                                float scale, __nv_bfloat16 *__restrict__ g, double *__restrict__ loss) {
  const long total = (long)B * kPix;
  double part = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long b = i / kPix, p = i % kPix;
    const int y = (int)(p / kW), x = (int)(p % kW);
    const bool interior = y > 0 && x > 0 && y < kH - 1 && x < kW - 1;
    __align__(16) __nv_bfloat16 c0[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      float gv = 0.f;
      if (c < 4 && interior) {
        const float d = pred[(b * 4 + c) * kPix + p] - tgt[(b * 4 + c) * kPix + p];
        part += (double)d * d;
        gv = 2.f * scale * d;
      }
      c0[c] = __float2bfloat16(gv);
    }
    *reinterpret_cast<uint4 *>(g + ((b * 2 + 0) * kPix + p) * 8) = *reinterpret_cast<const uint4 *>(c0);
    *reinterpret_cast<uint4 *>(g + ((b * 2 + 1) * kPix + p) * 8) = make_uint4(0, 0, 0, 0);
  }
  for (int m = 16; m >= 1; m >>= 1) part += __shfl_xor_sync(0xffffffffu, part, m);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, part * scale);
}

// Adam (FP32 master weights).
static __global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ gw, float *__restrict__ m,
                            float *__restrict__ v, long n, float lr, float b1, float b2, float eps,
                            float bc1, float bc2) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float g = gw[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

}  // namespace cnn
}  // namespace msfem
