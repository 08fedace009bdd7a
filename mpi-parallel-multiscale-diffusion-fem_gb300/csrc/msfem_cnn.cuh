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
//            cores (mma.sync m16n8k16 bf16, FP32 accumulators); FP32 master
//            weights and Adam; the weight gradient is an FP32 reduction.
//
// Device layouts: activations NHWC BF16 [B][33][33][C] with C padded to a
// multiple of 16 (first layer 16 channels, 3 used; last layer 16, 4 used).
// Weights for the forward pass [Cout][9][Cin], for the input-gradient pass
// (transposed, taps flipped) [Cin][9][Cout]; rows padded by 8 elements in
// shared memory so the fragment loads of one warp hit distinct banks.
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

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

// Epilogue modes of the convolution kernel.
enum { EPI_RELU_BF16 = 0,   // out = bf16(relu(acc + b))          (hidden layers)
       EPI_F32_NCHW = 1,    // out = float(acc + b), NCHW, real channels (last layer)
       EPI_MASK_BF16 = 2 }; // out = bf16(acc * [mask > 0])       (input gradient)

// 3x3 'same' convolution of one image per CTA as an implicit GEMM on the
// tensor cores: D[pixel][cout] = sum_{tap, cin} X[pixel + tap][cin] W[cout][tap][cin].
// X: [B][33][33][CIN] bf16, Wt: [COUT][9][CIN] bf16 (layout already chosen by
// the caller: forward weights or transposed/flipped ones).
template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(256)
conv3x3_kernel(const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ Wt,
               const float *__restrict__ bias, const __nv_bfloat16 *__restrict__ mask, void *out, int cout_real,
               int dil) {
  constexpr int SP = CIN + 8;           // smem pixel pitch (bf16)
  constexpr int WP = 9 * CIN + 8;       // smem weight row pitch (bf16)
  const int HP = kH + 2 * dil;          // halo tile side
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *s_in = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
  __nv_bfloat16 *s_w = s_in + HP * HP * SP;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const __nv_bfloat16 *xb = X + (long)b * kPix * CIN;
  // input tile with a zero halo (16-byte chunks)
  constexpr int CH = CIN / 8;
  for (int i = tid; i < HP * HP * CH; i += 256) {
    const int pix = i / CH, c8 = (i % CH) * 8;
    const int hy = pix / HP, hx = pix % HP;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (hy >= dil && hy < kH + dil && hx >= dil && hx < kW + dil)
      v = *reinterpret_cast<const uint4 *>(xb + ((hy - dil) * kW + (hx - dil)) * CIN + c8);
    *reinterpret_cast<uint4 *>(s_in + pix * SP + c8) = v;
  }
  for (int i = tid; i < COUT * 9 * CH; i += 256) {
    const int co = i / (9 * CH), r = i % (9 * CH);
    *reinterpret_cast<uint4 *>(s_w + co * WP + r * 8) = *reinterpret_cast<const uint4 *>(Wt + (long)co * 9 * CIN + r * 8);
  }
  __syncthreads();
  const int g = lane >> 2, t = lane & 3;
  constexpr int NT = COUT / 8;
  constexpr int MT = (kPix + 15) / 16;
  constexpr int MB = 3;  // m-tiles per warp pass: each weight fragment feeds MB x NT mma
  // ldmatrix.x4 row of this lane: pixel (lane & 15) of the m-tile, channel
  // offset (lane >> 4) * 8; pixels past the image read the (always zero) halo corner
  const uint32_t s_in_addr = (uint32_t)__cvta_generic_to_shared(s_in);
  for (int mt0 = warp * MB; mt0 < MT; mt0 += 8 * MB) {
    float acc[MB][NT][4];
    int rowbase[MB];
#pragma unroll
    for (int mb = 0; mb < MB; ++mb) {
#pragma unroll
      for (int n = 0; n < NT; ++n)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[mb][n][e] = 0.f;
      const int pr = (mt0 + mb) * 16 + (lane & 15);
      rowbase[mb] = pr < kPix ? (pr / kW) * HP + (pr % kW) : -1;
    }
#pragma unroll 1
    for (int tap = 0; tap < 9; ++tap) {
      const int toff = (tap / 3) * dil * HP + (tap % 3) * dil;
#pragma unroll
      for (int ks = 0; ks < CIN / 16; ++ks) {
        const int c0 = ks * 16 + 2 * t;
        uint32_t bfr[NT][2];
#pragma unroll
        for (int n = 0; n < NT; ++n) {
          const __nv_bfloat16 *wr = s_w + (n * 8 + g) * WP + tap * CIN + c0;
          bfr[n][0] = ld32(wr);
          bfr[n][1] = ld32(wr + 8);
        }
#pragma unroll
        for (int mb = 0; mb < MB; ++mb) {
          const int pix = rowbase[mb] >= 0 ? rowbase[mb] + toff : 0;
          const uint32_t addr = s_in_addr + (uint32_t)((pix * SP + ks * 16 + (lane >> 4) * 8) * 2);
          uint32_t a[4];
          asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                       : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3])
                       : "r"(addr));
#pragma unroll
          for (int n = 0; n < NT; ++n) mma_bf16(acc[mb][n], a, bfr[n]);
        }
      }
    }
    // epilogue: rows pa / pb of each m-tile, columns n*8 + 2t, +1
#pragma unroll
    for (int mb = 0; mb < MB; ++mb) {
      const int pa = (mt0 + mb) * 16 + g, pb = pa + 8;
#pragma unroll
      for (int n = 0; n < NT; ++n) {
        const int co = n * 8 + 2 * t;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int p = h ? pb : pa;
          if (p >= kPix) continue;
          float v0 = acc[mb][n][2 * h], v1 = acc[mb][n][2 * h + 1];
          if (EPI == EPI_RELU_BF16) {
            v0 = fmaxf(v0 + bias[co], 0.f);
            v1 = fmaxf(v1 + bias[co + 1], 0.f);
            __nv_bfloat16 *o = reinterpret_cast<__nv_bfloat16 *>(out) + ((long)b * kPix + p) * COUT + co;
            *reinterpret_cast<__nv_bfloat162 *>(o) = __floats2bfloat162_rn(v0, v1);
          } else if (EPI == EPI_F32_NCHW) {
            float *o = reinterpret_cast<float *>(out) + (long)b * cout_real * kPix + p;
            if (co < cout_real) o[(long)co * kPix] = v0 + bias[co];
            if (co + 1 < cout_real) o[(long)(co + 1) * kPix] = v1 + bias[co + 1];
          } else {
            const __nv_bfloat16 *mk = mask + ((long)b * kPix + p) * COUT + co;
            const float m0 = __bfloat162float(mk[0]) > 0.f ? 1.f : 0.f;
            const float m1 = __bfloat162float(mk[1]) > 0.f ? 1.f : 0.f;
            __nv_bfloat16 *o = reinterpret_cast<__nv_bfloat16 *>(out) + ((long)b * kPix + p) * COUT + co;
            *reinterpret_cast<__nv_bfloat162 *>(o) = __floats2bfloat162_rn(v0 * m0, v1 * m1);
          }
        }
      }
    }
  }
}

template <int CIN, int COUT>
constexpr size_t conv_smem(int dil) {
  return sizeof(__nv_bfloat16) * ((size_t)(kH + 2 * dil) * (kW + 2 * dil) * (CIN + 8) + (size_t)COUT * (9 * CIN + 8));
}

// Weight/bias gradient of one layer, FP32 accumulation:
//   dW[co][ci][tap] += sum_p G[p][co] X[p + tap][ci],  db[co] += sum_p G[p][co]
// G: [B][33][33][GC] bf16 (output gradient), X: [B][33][33][XC] bf16 (layer input).
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
    const __nv_bfloat16 *xb = X + (long)b * kPix * XC;
    const __nv_bfloat16 *gb = G + (long)b * kPix * GC;
    for (int i = tid; i < HP * HP * (XC / 8); i += 256) {
      const int pix = i / (XC / 8), c8 = (i % (XC / 8)) * 8;
      const int hy = pix / HP, hx = pix % HP;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (hy >= dil && hy < kH + dil && hx >= dil && hx < kW + dil)
        v = *reinterpret_cast<const uint4 *>(xb + ((hy - dil) * kW + (hx - dil)) * XC + c8);
      *reinterpret_cast<uint4 *>(s_x + pix * XC + c8) = v;
    }
    for (int i = tid; i < kPix * (GC / 8); i += 256)
      *reinterpret_cast<uint4 *>(s_g + i * 8) = *reinterpret_cast<const uint4 *>(gb + i * 8);
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
__global__ void pack_layer_kernel(const float *__restrict__ params, int layer, __nv_bfloat16 *__restrict__ wf,
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

// Features NCHW FP32 [B][3][33][33] -> NHWC BF16 [B][33][33][16].
__global__ void features_to_nhwc_kernel(const float *__restrict__ f, int B, __nv_bfloat16 *__restrict__ x) {
  const long total = (long)B * kPix;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long b = i / kPix, p = i % kPix;
    __nv_bfloat16 *o = x + i * 16;
#pragma unroll
    for (int c = 0; c < 16; ++c) o[c] = __float2bfloat16(c < 3 ? f[(b * 3 + c) * kPix + p] : 0.f);
  }
}

// MSE loss over interior nodes and its gradient (NHWC BF16, 16 channels).
__global__ void mse_loss_kernel(const float *__restrict__ pred, const float *__restrict__ tgt, int B,
                                float scale, __nv_bfloat16 *__restrict__ g, double *__restrict__ loss) {
  const long total = (long)B * kPix;
  double part = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long b = i / kPix, p = i % kPix;
    const int y = (int)(p / kW), x = (int)(p % kW);
    const bool interior = y > 0 && x > 0 && y < kH - 1 && x < kW - 1;
    __nv_bfloat16 *o = g + i * 16;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      float gv = 0.f;
      if (c < 4 && interior) {
        const float d = pred[(b * 4 + c) * kPix + p] - tgt[(b * 4 + c) * kPix + p];
        part += (double)d * d;
        gv = 2.f * scale * d;
      }
      o[c] = __float2bfloat16(gv);
    }
  }
  for (int m = 16; m >= 1; m >>= 1) part += __shfl_xor_sync(0xffffffffu, part, m);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, part * scale);
}

// Adam (FP32 master weights).
__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ gw, float *__restrict__ m,
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
