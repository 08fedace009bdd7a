// msfem_conv_tc.cuh -- the warm-start network's 3x3 dilated convolution on
// the 5th-generation tensor cores (sm_103a): TMA-staged input windows,
// tcgen05.mma BF16 x BF16 -> FP32 with the accumulators in tensor memory,
// tcgen05.ld epilogue.
//
// Implicit GEMM, D[position][cout] = sum_{tap, cin} X[position + tap][cin] W[cout][tap][cin]:
//   M = 128 output positions per MMA, N = COUT (32 or 16), K = 16 per MMA.
//
// Shifted windows instead of im2col.  Output positions run over a padded-
// width grid (33 rows x Wp = 33 + 2 d columns; columns >= 33 are computed and
// discarded), so the input pixel of position P under tap (ty, tx) sits at
// window index P - r0 Wp + ty d Wp + tx d: a constant shift per tap.  The
// window (input rows r0 - d ... with d zero columns either side, zero rows
// past the image) is loaded by TMA as one box per 8-channel block (a run of
// contiguous 16-byte pixels per row in the blocked global layout), whose shared-
// memory image [row][col][8 ch] is exactly the no-swizzle K-major canonical
// layout of the A operand: core matrix = 8 consecutive positions x 16 bytes,
// positions 16 B apart (SBO = 128 B), the next 8 channels one box further
// (LBO = box bytes).  A tap is then just a different descriptor start
// address.  Weights sit in the same layout, [k-block][cout][8].
//
// Work item = one image's segment of G = 4 tiles (512 positions).  A CTA of
// ten warps runs a two-stage pipeline over its items: a TMA producer, a
// single-thread MMA issuer and eight epilogue warps (warp w reads TMEM lanes
// 32 (w % 4)..+31, one position per thread), coupled by mbarriers, so the
// loads, the MMAs and the epilogue of consecutive items overlap.  Every wait
// is bounded (about 2 s); on a timeout the CTA records an error code, the
// other roles stop, in-flight copies get a bounded wait, TMEM is freed.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace msfem {
namespace cnn {
namespace tc {

constexpr int kTiles = 4;                        // 128-position tiles per work item
// Window rows per TMA box: 8 rows of wp pixels are 128 wp bytes, so every box
// of a window starts on a 128-byte boundary of shared memory (the alignment
// a tensor copy's destination needs); a second map carries the remainder.
constexpr int kBoxRows = 8;
constexpr uint64_t kWaitNs = 2000000000ull;      // bound of every wait

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (no swizzle, K-major canonical layout):
// start address, leading-dimension byte offset (next core matrix along K),
// stride byte offset (next 8 rows), all in 16-byte units; version 1 at bit 46.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Wait for the phase with the given parity; false after kWaitNs.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity) {
  if (mbar_try(a, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try(a, parity))
    if (global_ns() - t0 > kWaitNs) return false;
  return true;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(mbar)
      : "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(dst_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}
// 16 consecutive FP32 columns.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}

// Geometry of one layer's launch (host and device agree on it).
struct ConvGeom {
  int dil, wp, npos, tiles, segs, box_rows;
  uint32_t chunk_bytes, chunk_stride;
};
__host__ __device__ inline ConvGeom conv_geom(int dil) {
  ConvGeom g;
  g.dil = dil;
  g.wp = kW + 2 * dil;
  g.npos = kH * g.wp;
  g.tiles = (g.npos + 127) / 128;
  g.segs = (g.tiles + kTiles - 1) / kTiles;
  // window rows covering every read: position offset < wp plus 512 positions
  // plus the largest tap shift 2 d wp + 2 d (see the header comment)
  g.box_rows = (kTiles * 128 + 2 * dil * g.wp + 2 * dil + g.wp - 1) / g.wp + 1;
  g.chunk_bytes = (uint32_t)g.box_rows * g.wp * 16;
  g.chunk_stride = (g.chunk_bytes + 1023u) & ~1023u;
  return g;
}
template <int CIN, int COUT>
__host__ __device__ constexpr uint32_t weight_region() {
  return ((uint32_t)9 * CIN * COUT * 2 + 1023u) & ~1023u;
}
constexpr int kStages = 2;  // windows in shared memory and accumulator sets in TMEM
template <int CIN, int COUT>
__host__ inline size_t conv_tc_smem(int dil) {
  // + 1 KB to align the dynamic base to 1024 B
  return 1024 + weight_region<CIN, COUT>() + (size_t)kStages * (CIN / 8) * conv_geom(dil).chunk_stride;
}
constexpr int kEpiWarps = 8;                   // warps 0-7: epilogue (warp w: TMEM lane quarter w % 4)
constexpr int kThreads = 32 * (kEpiWarps + 2);  // warp 8: TMA producer, warp 9: MMA issuer

// A wait that also gives up when another role of the CTA has aborted.
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t a, uint32_t parity, volatile int *abort_flag) {
  if (mbar_try(a, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try(a, parity)) {
    if (*abort_flag) return false;
    if (global_ns() - t0 > kWaitNs) return false;
  }
  return true;
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(a) : "memory");
}

// X ([B][CIN/8][33][33][8] bf16) is described by xmap / xmap_rem as 8-byte
// elements, 3D: 66 per row (33 pixels x 16 B), 33 rows, B * CIN/8 channel
// blocks; boxes of 2 wp x kBoxRows x 1 (xmap) and 2 wp x (box_rows mod
// kBoxRows) x 1 (xmap_rem) starting at element -2 dil (zero-filled outside),
// so a box row is one contiguous run of wp pixels.
// Wt: [COUT][9][CIN] bf16.  Outputs: blocked BF16 (hidden layers, input
// gradients) or NCHW FP32 (prediction).  err: set to 1 (window load timed
// out), 2 (MMA side timed out) or 3 (epilogue side timed out).
//
// Roles (320 threads): warp 8 lane 0 streams windows into kStages buffers
// (full[s] <- TMA bytes; waits empty[s]); warp 9 lane 0 issues the MMAs of
// item i into accumulator set i % kStages (waits full[s] and accumulator
// drained acce[s]; commits to empty[s] and accf[s]); warps 0-7 drain the
// accumulators (wait accf[s], tcgen05.ld, stores, arrive acce[s]).  Item i of
// a CTA uses stage s = i % 2 for the u = i / 2-th time: phase parity u & 1.
template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(kThreads, 2)
conv3x3_tc_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap xmap_rem,
                  const __nv_bfloat16 *__restrict__ Wt,
                  const float *__restrict__ bias, const __nv_bfloat16 *__restrict__ mask, void *out, int cout_real,
                  int dil, int B, int *err) {
  static_assert(CIN % 16 == 0 && (COUT == 16 || COUT == 32), "shapes");
  constexpr int KC = CIN / 8;                          // 8-channel k-blocks per tap
  constexpr uint32_t NACC = kTiles * COUT;             // TMEM columns per accumulator set
  constexpr uint32_t NCOL = kStages * NACC;            // 256 or 128
  constexpr uint32_t IDESC = idesc_bf16(128, COUT);
  constexpr uint32_t WREG = weight_region<CIN, COUT>();
  extern __shared__ __align__(16) unsigned char smem_dyn[];
  __shared__ __align__(8) uint64_t bar_full[kStages], bar_empty[kStages], bar_accf[kStages], bar_acce[kStages];
  __shared__ uint32_t tmem_base;
  __shared__ int abort_code;
  __shared__ float s_bias[COUT];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const ConvGeom g = conv_geom(dil);
  const long items = (long)B * g.segs;
  const uint32_t raw = smem_u32(smem_dyn);
  const uint32_t s_w = (raw + 1023u) & ~1023u;
  unsigned char *w_gen = smem_dyn + (s_w - raw);
  const uint32_t s_x = s_w + WREG;
  const uint32_t stage_bytes = KC * g.chunk_stride;
  volatile int *abort_v = &abort_code;
  if (tid < COUT) s_bias[tid] = bias != nullptr ? bias[tid] : 0.f;

  // weights -> [k-block = tap * KC + c8][cout][8 channels]
  for (int i = tid; i < COUT * 9 * KC; i += kThreads) {
    const int n = i / (9 * KC), kb = i % (9 * KC);
    const uint4 v = *reinterpret_cast<const uint4 *>(Wt + (long)n * 9 * CIN + kb * 8);
    *reinterpret_cast<uint4 *>(w_gen + (size_t)kb * (COUT * 16) + n * 16) = v;
  }
  if (tid == 0) {
    for (int st = 0; st < kStages; ++st) {
      mbar_init(smem_u32(&bar_full[st]), 1);
      mbar_init(smem_u32(&bar_empty[st]), 1);
      mbar_init(smem_u32(&bar_accf[st]), 1);
      mbar_init(smem_u32(&bar_acce[st]), kEpiWarps);
    }
    abort_code = 0;
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(smem_u32(&tmem_base), NCOL);
  fence_proxy_async();  // generic-proxy weight stores -> tensor-core reads
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tbase = tmem_base;

  if (warp == kEpiWarps) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      long it = blockIdx.x;
      int i = 0;
      for (; it < items; it += gridDim.x, ++i) {
        const int st = i % kStages, u = i / kStages;
        if (u > 0 && !mbar_wait_or_abort(smem_u32(&bar_empty[st]), (u - 1) & 1, abort_v)) {
          if (!*abort_v) { abort_code = 1; atomicExch(err, 1); }
          // the copies already issued must land before the CTA's smem goes
          for (int j = max(0, i - kStages); j < i; ++j)
            mbar_wait(smem_u32(&bar_full[j % kStages]), (j / kStages) & 1);
          break;
        }
        const int b = (int)(it / g.segs), seg = (int)(it % g.segs);
        const int r0 = (seg * kTiles * 128) / g.wp;
        const uint32_t full = smem_u32(&bar_full[st]);
        mbar_expect_tx(full, KC * g.chunk_bytes);
        // per 8-channel block: boxes of kBoxRows rows (several in flight) and
        // one box of the remaining rows; every destination is a multiple of
        // 128 B from the 1024-aligned block start
        const int nfull = g.box_rows / kBoxRows, rem = g.box_rows - nfull * kBoxRows;
        for (int k = 0; k < KC; ++k) {
          const uint32_t dst = s_x + st * stage_bytes + k * g.chunk_stride;
          for (int q = 0; q < nfull; ++q)
            tma_load_3d(dst + (uint32_t)(q * kBoxRows * g.wp * 16), &xmap, -2 * dil, r0 - dil + q * kBoxRows,
                        b * KC + k, full);
          if (rem > 0)
            tma_load_3d(dst + (uint32_t)(nfull * kBoxRows * g.wp * 16), &xmap_rem, -2 * dil,
                        r0 - dil + nfull * kBoxRows, b * KC + k, full);
        }
      }
    }
  } else if (warp == kEpiWarps + 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      // base descriptors and the per-tap shift of the A start address
      const uint64_t a_desc0 = smem_desc(s_x, g.chunk_stride, 128);
      const uint64_t b_desc0 = smem_desc(s_w, COUT * 16, 128);
      const uint32_t a_kstep = (2 * g.chunk_stride) >> 4;  // next 16 channels
      uint32_t tap_off[9];
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) tap_off[tap] = (uint32_t)((tap / 3) * dil * g.wp + (tap % 3) * dil);
      long it = blockIdx.x;
      int i = 0;
      for (; it < items; it += gridDim.x, ++i) {
        const int st = i % kStages, u = i / kStages;
        if (!mbar_wait_or_abort(smem_u32(&bar_full[st]), u & 1, abort_v) ||
            (u > 0 && !mbar_wait_or_abort(smem_u32(&bar_acce[st]), (u - 1) & 1, abort_v))) {
          if (!*abort_v) { abort_code = 2; atomicExch(err, 2); }
          break;
        }
        fence_after_sync();
        const int seg = (int)(it % g.segs);
        const int p0 = seg * kTiles * 128, r0 = p0 / g.wp;
        const int nt = min(kTiles, g.tiles - seg * kTiles);  // tiles holding real positions
        // descriptors advance in 16-byte units: one window position is 16 B
        const uint64_t a_item = a_desc0 + (uint64_t)((st * stage_bytes) >> 4);
        for (int t = 0; t < nt; ++t) {
          const uint32_t d = tbase + (uint32_t)(st * NACC + t * COUT);
          const uint64_t a_t = a_item + (uint64_t)(p0 + t * 128 - r0 * g.wp);
#pragma unroll
          for (int tap = 0; tap < 9; ++tap) {
#pragma unroll
            for (int ks = 0; ks < CIN / 16; ++ks)
              umma_bf16(d, a_t + (uint64_t)(tap_off[tap] + ks * a_kstep),
                        b_desc0 + (uint64_t)((tap * KC + 2 * ks) * COUT), IDESC, (tap | ks) != 0 ? 1u : 0u);
          }
        }
        umma_commit(smem_u32(&bar_empty[st]));  // the window may be overwritten
        umma_commit(smem_u32(&bar_accf[st]));   // the accumulators are ready
      }
      // the last commits must land before TMEM is released
      if (i > 0) {
        const int last = i - 1;
        mbar_wait(smem_u32(&bar_accf[last % kStages]), (last / kStages) & 1);
      }
    }
  } else {
    // ---------------- epilogue: warps 0-7 ----------------
    // warp w reads TMEM lanes 32 (w % 4) .. +31 (the quarter its position in
    // the warpgroup allows) of tiles w / 4 and w / 4 + 2: both loads in
    // flight before one wait
    const int q = warp & 3, h = warp >> 2;
    auto store = [&](const uint32_t (&v)[COUT], int b, int pos) {
      const int y = pos / g.wp, xp = pos - (pos / g.wp) * g.wp;
      const int pix = y * kW + xp;
      if (pos >= g.npos || xp >= kW) {
        // a padding column or a position past the image: computed, not stored
      } else if constexpr (EPI == EPI_RELU_BF16) {
        // channel block c / 8 of pixel pix: 16 contiguous bytes, lanes adjacent
        __nv_bfloat16 *o = reinterpret_cast<__nv_bfloat16 *>(out) + ((long)b * (COUT / 8) * kPix + pix) * 8;
#pragma unroll
        for (int c = 0; c < COUT; c += 8) {
          __align__(16) __nv_bfloat162 hh[4];
#pragma unroll
          for (int j = 0; j < 4; ++j)
            hh[j] = __floats2bfloat162_rn(fmaxf(__uint_as_float(v[c + 2 * j]) + s_bias[c + 2 * j], 0.f),
                                          fmaxf(__uint_as_float(v[c + 2 * j + 1]) + s_bias[c + 2 * j + 1], 0.f));
          *reinterpret_cast<uint4 *>(o + (long)(c / 8) * kPix * 8) = *reinterpret_cast<const uint4 *>(hh);
        }
      } else if constexpr (EPI == EPI_F32_NCHW) {
        float *o = reinterpret_cast<float *>(out) + (long)b * cout_real * kPix + pix;
#pragma unroll
        for (int c = 0; c < COUT; ++c)
          if (c < cout_real) o[(long)c * kPix] = __uint_as_float(v[c]) + s_bias[c];
      } else {
        const long base = ((long)b * (COUT / 8) * kPix + pix) * 8;
        const __nv_bfloat16 *mk = mask + base;
        __nv_bfloat16 *o = reinterpret_cast<__nv_bfloat16 *>(out) + base;
#pragma unroll
        for (int c = 0; c < COUT; c += 8) {
          const uint4 mraw = *reinterpret_cast<const uint4 *>(mk + (long)(c / 8) * kPix * 8);
          const __nv_bfloat16 *m8 = reinterpret_cast<const __nv_bfloat16 *>(&mraw);
          __align__(16) __nv_bfloat162 hh[4];
#pragma unroll
          for (int j = 0; j < 4; ++j)
            hh[j] = __floats2bfloat162_rn(
                __bfloat162float(m8[2 * j]) > 0.f ? __uint_as_float(v[c + 2 * j]) : 0.f,
                __bfloat162float(m8[2 * j + 1]) > 0.f ? __uint_as_float(v[c + 2 * j + 1]) : 0.f);
          *reinterpret_cast<uint4 *>(o + (long)(c / 8) * kPix * 8) = *reinterpret_cast<const uint4 *>(hh);
        }
      }
    };
    long it = blockIdx.x;
    int i = 0;
    for (; it < items; it += gridDim.x, ++i) {
      const int st = i % kStages, u = i / kStages;
      // warp-uniform decision: tcgen05.ld below is a warp-collective instruction
      const bool ok = __all_sync(0xffffffffu, mbar_wait_or_abort(smem_u32(&bar_accf[st]), u & 1, abort_v));
      if (!ok) {
        if (lane == 0 && !*abort_v) { abort_code = 3; atomicExch(err, 3); }
        break;
      }
      fence_after_sync();
      const int b = (int)(it / g.segs), seg = (int)(it % g.segs);
      const int p0 = seg * kTiles * 128;
      const int nt = min(kTiles, g.tiles - seg * kTiles);
      const bool has0 = h < nt, has1 = h + 2 < nt;  // warp-uniform
      const uint32_t ta = tbase + ((uint32_t)(q * 32) << 16) + (uint32_t)(st * NACC);
      uint32_t va[COUT], vb[COUT];
      if (has0) {
        if constexpr (COUT == 32) tmem_ld32(ta + (uint32_t)(h * COUT), va);
        else tmem_ld16(ta + (uint32_t)(h * COUT), va);
      }
      if (has1) {
        if constexpr (COUT == 32) tmem_ld32(ta + (uint32_t)((h + 2) * COUT), vb);
        else tmem_ld16(ta + (uint32_t)((h + 2) * COUT), vb);
      }
      tmem_wait_ld();
      if (has0) store(va, b, p0 + h * 128 + q * 32 + lane);
      if (has1) store(vb, b, p0 + (h + 2) * 128 + q * 32 + lane);
      // accumulator set st drained by this warp
      fence_before_sync();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&bar_acce[st]));
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) tmem_dealloc(tbase, NCOL);
}

// ---------------------------------------------------------------------------
// Weight and bias gradient on the tensor cores.
//
//   dW[cout][cin][tap] = sum_{b, p} G[b][p][cout] X[b][p + shift(tap)][cin],
//   db[cout]           = sum_{b, p} G[b][p][cout],
//
// a GEMM per tap with K = the output positions of all images: D_tap(M x N)
// += A(M x 16) B_tap(16 x N) per 16 positions, M = 128 rows of output
// channels (GC real, the rest zero), N = XC input channels.  Both operands
// are read MN-major straight from the channel-blocked layout (8 channels =
// 16 contiguous bytes per position): B_tap is the TMA-loaded input window of
// the forward pass (same tensor map geometry), the tap a shift of its start
// address; A is the output gradient staged per 16 positions into 16 groups of
// 8 channels, the groups beyond GC zero.  The bias gradient is one more
// accumulator against a tile of ones.  Positions run over the forward pass's
// padded-width grid, where G is zero outside the image, so every product of
// the forward convolution appears exactly once.
//
// A CTA accumulates its items (image, 256 positions) in TMEM (9 + 1
// accumulators of N columns) and adds them to dW/db with FP32 atomics at the
// end.  Per item: TMA window + staged G -> one thread issues 16 x 10 MMAs ->
// commit; every wait is bounded (err 1: window load, 2: MMA).
// ---------------------------------------------------------------------------
constexpr int kWgPos = 256;                              // positions (K) per item
constexpr int kWgKsteps = kWgPos / 16;
constexpr int kWgThreads = 256;
constexpr uint32_t kWgKstepBytes = 16u * 256u;           // 16 channel groups x 16 positions x 16 B
constexpr uint32_t kWgStaging = (uint32_t)kWgKsteps * kWgKstepBytes;  // 64 KB
constexpr uint32_t kWgOnes = 1024u;                      // ones tile: up to 4 groups x 16 positions x 16 B

struct WgGeom {
  int dil, wp, npos, segs, box_rows;
  uint32_t chunk_bytes, chunk_stride;
};
__host__ __device__ inline WgGeom wg_geom(int dil) {
  WgGeom g;
  g.dil = dil;
  g.wp = kW + 2 * dil;
  g.npos = kH * g.wp;
  g.segs = (g.npos + kWgPos - 1) / kWgPos;
  g.box_rows = (kWgPos + 2 * dil * g.wp + 2 * dil + g.wp - 1) / g.wp + 1;
  g.chunk_bytes = (uint32_t)g.box_rows * g.wp * 16;
  g.chunk_stride = (g.chunk_bytes + 1023u) & ~1023u;
  return g;
}
template <int XC>
__host__ inline size_t wgrad_tc_smem(int dil) {
  return 1024 + kWgStaging + kWgOnes + (size_t)(XC / 8) * wg_geom(dil).chunk_stride;
}
template <int XC>
__host__ __device__ constexpr uint32_t wgrad_tmem_cols() {
  return 10 * XC <= 256 ? 256u : 512u;
}

template <int XC, int GC>
__global__ void __launch_bounds__(kWgThreads, 1)
conv3x3_wgrad_tc_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap xmap_rem,
                        const __nv_bfloat16 *__restrict__ G, int B, int cin_real, int cout_real,
                        float *__restrict__ dW, float *__restrict__ db, int dil, int *err) {
  static_assert((XC == 16 || XC == 32) && (GC == 16 || GC == 32), "shapes");
  constexpr int KC = XC / 8, GB = GC / 8;
  constexpr uint32_t N = XC;
  // A and B MN-major (bits 15, 16), M = 128, N = XC
  constexpr uint32_t IDESC = idesc_bf16(128, N) | (1u << 15) | (1u << 16);
  constexpr uint32_t NCOL = wgrad_tmem_cols<XC>();
  extern __shared__ __align__(16) unsigned char smem_dyn[];
  __shared__ __align__(8) uint64_t bar_tma, bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_code;
  const int tid = threadIdx.x, warp = tid >> 5;
  const WgGeom g = wg_geom(dil);
  const uint32_t raw = smem_u32(smem_dyn);
  const uint32_t s_stage = (raw + 1023u) & ~1023u;
  const uint32_t s_ones = s_stage + kWgStaging;
  const uint32_t s_x = s_ones + kWgOnes;
  unsigned char *gen_stage = smem_dyn + (s_stage - raw);
  unsigned char *gen_ones = gen_stage + kWgStaging;
  // zero staging (its groups >= GC/8 stay zero: the padding rows of M = 128)
  for (uint32_t i = tid; i < kWgStaging / 16; i += kWgThreads)
    *reinterpret_cast<uint4 *>(gen_stage + 16 * i) = make_uint4(0, 0, 0, 0);
  for (uint32_t i = tid; i < kWgOnes / 4; i += kWgThreads)
    reinterpret_cast<uint32_t *>(gen_ones)[i] = 0x3F803F80u;  // bf16 1.0, 1.0
  if (tid == 0) {
    mbar_init(smem_u32(&bar_tma), 1);
    mbar_init(smem_u32(&bar_mma), 1);
    abort_code = 0;
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(smem_u32(&tmem_base), NCOL);
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tbase = tmem_base;
  uint32_t tap_off[9];
#pragma unroll
  for (int tap = 0; tap < 9; ++tap) tap_off[tap] = (uint32_t)((tap / 3) * dil * g.wp + (tap % 3) * dil);

  const long items = (long)B * g.segs;
  uint32_t phase = 0;
  bool first = true;
  bool tma_pending = false;
  for (long it = blockIdx.x; it < items; it += gridDim.x) {
    const int b = (int)(it / g.segs), seg = (int)(it % g.segs);
    const int p0 = seg * kWgPos, r0 = p0 / g.wp;
    if (tid == 0) {
      // the input window, as in the forward pass: boxes of kBoxRows rows (128 wp
      // bytes each, 128-byte aligned destinations) and the remainder
      const uint32_t full = smem_u32(&bar_tma);
      mbar_expect_tx(full, KC * g.chunk_bytes);
      const int nfull = g.box_rows / kBoxRows, rem = g.box_rows - nfull * kBoxRows;
      for (int k = 0; k < KC; ++k) {
        const uint32_t dst = s_x + k * g.chunk_stride;
        for (int q = 0; q < nfull; ++q)
          tma_load_3d(dst + (uint32_t)(q * kBoxRows * g.wp * 16), &xmap, -2 * dil, r0 - dil + q * kBoxRows,
                      b * KC + k, full);
        if (rem > 0)
          tma_load_3d(dst + (uint32_t)(nfull * kBoxRows * g.wp * 16), &xmap_rem, -2 * dil,
                      r0 - dil + nfull * kBoxRows, b * KC + k, full);
      }
      tma_pending = true;
    }
    // the output gradient of the item's positions: [k-step][group][16 positions][8 ch]
    for (int i = tid; i < kWgPos * GB; i += kWgThreads) {
      const int grp = i / kWgPos, r = i - grp * kWgPos;
      const int P = p0 + r, y = P / g.wp, x = P - y * g.wp;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (y < kH && x < kW)
        v = *reinterpret_cast<const uint4 *>(G + (((long)b * GB + grp) * kPix + y * kW + x) * 8);
      *reinterpret_cast<uint4 *>(gen_stage + (r >> 4) * kWgKstepBytes + grp * 256 + (r & 15) * 16) = v;
    }
    fence_proxy_async();  // generic-proxy staging stores -> tensor-core reads
    __syncthreads();
    if (tid == 0) {
      if (!mbar_wait(smem_u32(&bar_tma), phase)) {
        abort_code = 1;
        atomicExch(err, 1);
      } else {
        tma_pending = false;
        fence_after_sync();
        const uint32_t pos0 = (uint32_t)(p0 - r0 * g.wp);  // item start within the window's first row
        // MN-major operands: LBO = stride of the 8-row groups along K (the next
        // 8 positions, 128 B), SBO = stride of the 8-channel groups along M/N
        const uint64_t ones = smem_desc(s_ones, 128, 256);
#pragma unroll 1
        for (int ks = 0; ks < kWgKsteps; ++ks) {
          const uint64_t a = smem_desc(s_stage + ks * kWgKstepBytes, 128, 256);
          const uint32_t acc = (first && ks == 0) ? 0u : 1u;
          const uint32_t xs = s_x + (pos0 + 16u * ks) * 16u;
#pragma unroll
          for (int tap = 0; tap < 9; ++tap)
            umma_bf16(tbase + tap * N, a, smem_desc(xs + tap_off[tap] * 16u, 128, g.chunk_stride), IDESC, acc);
          umma_bf16(tbase + 9 * N, a, ones, IDESC, acc);
        }
        umma_commit(smem_u32(&bar_mma));
        if (!mbar_wait(smem_u32(&bar_mma), phase)) {
          abort_code = 2;
          atomicExch(err, 2);
        }
      }
    }
    __syncthreads();
    if (abort_code) break;
    phase ^= 1u;
    first = false;
  }
  // a window copy still in flight must land before the CTA's smem goes, and
  // MMAs still running before their TMEM is released
  if (tid == 0 && tma_pending) mbar_wait(smem_u32(&bar_tma), phase);
  if (tid == 0 && abort_code == 2) mbar_wait(smem_u32(&bar_mma), phase);
  fence_after_sync();
  if (!abort_code && !first && warp == 0) {
    // rows (output channels) 0..31 sit in TMEM lanes 0..31: warp 0's quarter
    const int co = threadIdx.x;
    uint32_t v[32];
#pragma unroll 1
    for (int t = 0; t < 10; ++t) {
      if constexpr (N == 32) {
        tmem_ld32(tbase + t * N, v);
      } else {
        uint32_t h[16];
        tmem_ld16(tbase + t * N, h);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = h[j];
      }
      tmem_wait_ld();
      if (co < cout_real) {
        if (t < 9) {
#pragma unroll
          for (int ci = 0; ci < (int)N; ++ci)
            if (ci < cin_real) atomicAdd(dW + ((long)co * cin_real + ci) * 9 + t, __uint_as_float(v[ci]));
        } else {
          atomicAdd(db + co, __uint_as_float(v[0]));
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) tmem_dealloc(tbase, NCOL);
}

}  // namespace tc
}  // namespace cnn
}  // namespace msfem
