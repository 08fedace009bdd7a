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
//            msfem_conv_tc.cuh); FP32 master weights and Adam; the weight
//            gradient is an FP32 reduction on the CUDA cores.
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

// Weight/bias gradient of one layer, FP32 accumulation:
//   dW[co][ci][tap] += sum_p G[p][co] X[p + tap][ci],  db[co] += sum_p G[p][co]
// G: output gradient, GC channels; X: layer input, XC channels; both in the
// channel-blocked layout [B][C/8][33][33][8] bf16.
// Thread = (ci, 4 output channels); CTAs stride over the images.
template <int XC, int GC>
__global__ void __launch_bounds__(256)
conv3x3_wgrad_kernel(const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ G, int B,
                     int cin_real, int cout_real, float *__restrict__ dW, float *__restrict__ db, int dil) {
  const int HP = kH + 2 * dil;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *s_x = reinterpret_cast<__nv_bfloat16 *>(smem_raw);   // [HP*HP][XC]
  __nv_bfloat16 *s_g = s_x + HP * HP * XC;                              // [kPix][GC]
  const int tid = threadIdx.x;
  const int ngrp = (cout_real + 3) / 4;
  const int ci = tid % 32, grp = tid / 32;  // 8 groups of 4 output channels
  const bool act = ci < cin_real && grp < ngrp;
  float acc[4][9], accb[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    accb[j] = 0.f;
#pragma unroll
    for (int tp = 0; tp < 9; ++tp) acc[j][tp] = 0.f;
  }
  for (int b = blockIdx.x; b < B; b += gridDim.x) {
    __syncthreads();
    const __nv_bfloat16 *xb = X + (long)b * kPix * XC;  // blocked: [XC/8][33][33][8]
    const __nv_bfloat16 *gb = G + (long)b * kPix * GC;
    for (int i = tid; i < HP * HP * (XC / 8); i += 256) {
      const int k = i / (HP * HP), pix = i % (HP * HP);
      const int hy = pix / HP, hx = pix % HP;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (hy >= dil && hy < kH + dil && hx >= dil && hx < kW + dil)
        v = *reinterpret_cast<const uint4 *>(xb + ((long)k * kPix + (hy - dil) * kW + (hx - dil)) * 8);
      *reinterpret_cast<uint4 *>(s_x + pix * XC + k * 8) = v;
    }
    for (int i = tid; i < kPix * (GC / 8); i += 256) {
      const int k = i / kPix, pix = i % kPix;
      *reinterpret_cast<uint4 *>(s_g + pix * GC + k * 8) =
          *reinterpret_cast<const uint4 *>(gb + ((long)k * kPix + pix) * 8);
    }
    __syncthreads();
    if (act) {
      const int co0 = grp * 4;
      for (int p = 0; p < kPix; ++p) {
        const int y = p / kW, x = p % kW;
        float gv[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) gv[j] = (co0 + j < cout_real) ? __bfloat162float(s_g[p * GC + co0 + j]) : 0.f;
#pragma unroll
        for (int tp = 0; tp < 9; ++tp) {
          const float xv = __bfloat162float(s_x[((y + (tp / 3) * dil) * HP + x + (tp % 3) * dil) * XC + ci]);
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[j][tp] = fmaf(gv[j], xv, acc[j][tp]);
        }
        if (ci == 0)
#pragma unroll
          for (int j = 0; j < 4; ++j) accb[j] += gv[j];
      }
    }
  }
  if (act) {
    const int co0 = grp * 4;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (co0 + j >= cout_real) continue;
#pragma unroll
      for (int tp = 0; tp < 9; ++tp) atomicAdd(dW + ((long)(co0 + j) * cin_real + ci) * 9 + tp, acc[j][tp]);
      if (ci == 0) atomicAdd(db + co0 + j, accb[j]);
    }
  }
}

template <int XC, int GC>
constexpr size_t wgrad_smem(int dil) {
  return sizeof(__nv_bfloat16) * ((size_t)(kH + 2 * dil) * (kW + 2 * dil) * XC + (size_t)kPix * GC);
}

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
