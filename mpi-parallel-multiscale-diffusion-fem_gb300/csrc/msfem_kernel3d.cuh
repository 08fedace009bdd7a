// msfem_kernel3d.cuh -- 3D multiscale-basis kernels for sm_103a.
//
// Same algorithm as the 2D kernels (diffusion_problem_basis.tpp:159-285):
// QGauss(2) trilinear Q1 assembly into a 27-point node stencil (8-colour
// scatter, no atomics), symmetric D^-1/2 scaling, all 8 Dirichlet problems
// (coarse trilinear nodal functions, basis_q1.tpp:50-75) advanced together by
// CG with per-RHS relative stopping, and the M = phi^T A phi / F = phi^T b
// epilogue.  FP64 form and mixed form (FP32 inner CG, FP64 residual
// refinement) as in 2D.
//
// A 3D local problem with 8 right-hand sides does not fit one SM's shared
// memory (N = 24: 15625 nodes x 176 B in FP64), so each persistent CTA owns
// a slot of a global-memory workspace: FP64 arrays structure-of-arrays
// ([component][node], coalesced along x), the mixed form's inner FP32 CG
// vectors node-major ([node][8 RHS], two 16-byte loads per neighbour).  The
// working set of one sweep (three node planes) stays in L1.  Bound: the FP64
// pipe in the FP64 form (26 FMA x 8 RHS per node per iteration against
// ~100 B of couplings), L1 throughput in the FP32 inner loop.
//
// Node (ix,iy,iz) of the (N+1)^3 grid sits at g = ((iz+1) P + iy + 1) P + ix + 1,
// P = N + 3 (a zero ring around the grid).  Each node stores its 13 "forward"
// couplings (offsets lexicographically after it); the 13 backward ones are
// the forward couplings of the neighbours.
#pragma once

#include <cooperative_groups.h>

#include "msfem_common.cuh"

namespace msfem {

constexpr int kNMax3D = MSFEM_MAX_N_3D;

// Per-slot workspace layout (in units of G = P^3 values, P = NMAX + 3).
struct Work3D {
  static constexpr int P = kNMax3D + 3;
  static constexpr long G = (long)P * P * P;
  // FP64 arrays
  static constexpr long kC64 = 0;              // [13][G] scaled couplings
  static constexpr long kD64 = kC64 + 13 * G;  // [G] diagonal
  static constexpr long kX64 = kD64 + G;       // [8][G] phi~ (boundary g~, interior x~)
  static constexpr long kR64 = kX64 + 8 * G;   // [8][G] residual (FP64 CG) / scratch
  static constexpr long kP64 = kR64 + 8 * G;   // [8][G] search direction (FP64 CG)
  static constexpr long kQ64 = kP64 + 8 * G;   // [8][G] A p
  static constexpr long kEnd64 = kQ64 + 8 * G;
  // FP32 arrays (mixed form): couplings [13][G], then the inner loop's
  // node-major vectors [G][8] from a 16-byte boundary (G rounded up to G4)
  static constexpr long G4 = (G + 3) & ~3L;
  static constexpr long kC32 = 0;               // [13][G]
  static constexpr long kD32 = kC32 + 13 * G4;  // [G][8] correction d
  static constexpr long kR32 = kD32 + 8 * G4;   // [G][8] residual
  static constexpr long kP32 = kR32 + 8 * G4;   // [G][8] search direction
  static constexpr long kQ32 = kP32 + 8 * G4;   // [G][8] A p
  static constexpr long kEnd32 = kQ32 + 8 * G4;
  // every slot starts on a 256-byte boundary (slot k at k * bytes())
  static constexpr size_t bytes(bool mixed) {
    return (sizeof(double) * kEnd64 + (mixed ? sizeof(float) * kEnd32 : 0) + 511) & ~size_t(255);
  }
  static_assert((sizeof(double) * kEnd64) % 16 == 0, "FP32 arrays start aligned");
};

// Forward offsets: (1,0,0), (-1..1,1,0), (-1..1,-1..1,1).
__device__ __forceinline__ void fwd_offset(int o, int &dx, int &dy, int &dz) {
  if (o == 0) { dx = 1; dy = 0; dz = 0; }
  else if (o < 4) { dx = o - 2; dy = 1; dz = 0; }
  else { const int m = o - 4; dx = m % 3 - 1; dy = m / 3 - 1; dz = 1; }
}
__device__ __forceinline__ int fwd_index(int dx, int dy, int dz) {
  if (dz == 1) return 4 + (dy + 1) * 3 + (dx + 1);
  if (dy == 1) return 1 + (dx + 1);
  return 0;  // (1,0,0)
}
__device__ __forceinline__ bool is_forward(int dx, int dy, int dz) {
  return dz > 0 || (dz == 0 && (dy > 0 || (dy == 0 && dx > 0)));
}

struct CellShared3D {
  double corners[24];
  double q1coef[64];
  double q1shift[3];
  double q1iscale;
  double jinv[9];      // affine: inverse fine Jacobian (row-major)
  double jfine[9];     // affine: fine Jacobian, column a = dx/dxi_a
  double absdet;
  double tmpl[8][36];  // affine scalar coefficient: K = sum_q a_q tmpl[q] (upper triangle)
  double bb[8];
  double bthr[8];      // stopping scale: ||b_i||^2 (relative tolerance) or 1 (absolute)
  double nu[8];
  double rho[8];
  double alpha[8];
  double beta[8];
  double dmin;
  int active[8];
  int iters[8];
  int inner_iters[8];  // mixed form: inner FP32 iterations per RHS
  float seg_thr[8];    // mixed form: stopping threshold on r.r of the current segment
  float seg_rho[2][8]; // mixed form: r.r of the current and next inner iteration
  float seg_beta[8];   // mixed form, slab cluster shape: beta of the next inner iteration
  int offs[13];        // grid offsets of the forward couplings
  int status;
  int affine;
  int need_nu;
  int done;
  int cell;
  int refinements;
};

__device__ __forceinline__ void trilinear_map(const double *cr, const double *t, double *x) {
  x[0] = x[1] = x[2] = 0.0;
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    const double w = ((v & 1) ? t[0] : 1.0 - t[0]) * ((v & 2) ? t[1] : 1.0 - t[1]) *
                     ((v & 4) ? t[2] : 1.0 - t[2]);
#pragma unroll
    for (int a = 0; a < 3; ++a) x[a] = fma(w, cr[3 * v + a], x[a]);
  }
}

__device__ __forceinline__ double gp3(int i) {
  return i ? 0.78867513459481288225457439025098 : 0.21132486540518711774542560974902;
}
__device__ __forceinline__ double lv3(int b, int q) { return b ? gp3(q) : gp3(1 - q); }

// reference gradient of vertex k at Gauss point q (component a)
__device__ __forceinline__ double rgrad(int k, int q, int a) {
  double g = ((k >> a) & 1) ? 1.0 : -1.0;
#pragma unroll
  for (int c = 0; c < 3; ++c)
    if (c != a) g *= lv3((k >> c) & 1, (q >> c) & 1);
  return g;
}

__device__ __forceinline__ int tri_index(int i, int j) {  // i <= j < 8
  return i * 8 - i * (i - 1) / 2 + (j - i);
}

// Element matrix (upper triangle, 36 entries) of fine cell (cx,cy,cz).
__device__ inline bool element3d(const KernelParams &p, const CellShared3D &cs, const double *__restrict__ tab,
                          int N, int cx, int cy, int cz, bool scalar, bool need_x, double (&K)[36]) {
  const int nfc = N * N * N, fc = cx + N * (cy + N * cz);
#pragma unroll
  for (int e = 0; e < 36; ++e) K[e] = 0.0;
  if (cs.affine && scalar) {
#pragma unroll 1
    for (int q = 0; q < 8; ++q) {
      double xq[3] = {0.0, 0.0, 0.0}, A[6];
      if (need_x) {
        const double u[3] = {cx + gp3(q & 1), cy + gp3((q >> 1) & 1), cz + gp3(q >> 2)};
#pragma unroll
        for (int a = 0; a < 3; ++a)
          xq[a] = cs.corners[a] + cs.jfine[3 * a] * u[0] + cs.jfine[3 * a + 1] * u[1] + cs.jfine[3 * a + 2] * u[2];
      }
      coef_at<3>(p, xq, tab, q, nfc, fc, A);
      const double a = A[0];
#pragma unroll
      for (int e = 0; e < 36; ++e) K[e] = fma(a, cs.tmpl[q][e], K[e]);
    }
    return true;
  }
  // general path: per-Gauss-point Jacobian and tensor coefficient
  const double invN = 1.0 / (double)N;
  double V[24];
#pragma unroll 1
  for (int k = 0; k < 8; ++k) {
    const double t[3] = {(cx + (k & 1)) * invN, (cy + ((k >> 1) & 1)) * invN, (cz + (k >> 2)) * invN};
    trilinear_map(cs.corners, t, V + 3 * k);
  }
  bool ok = true;
#pragma unroll 1
  for (int q = 0; q < 8; ++q) {
    double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, xq[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 8; ++k) {
      const double psi = lv3(k & 1, q & 1) * lv3((k >> 1) & 1, (q >> 1) & 1) * lv3(k >> 2, q >> 2);
      for (int a = 0; a < 3; ++a) {
        xq[a] += psi * V[3 * k + a];
        for (int c = 0; c < 3; ++c) J[3 * a + c] += V[3 * k + a] * rgrad(k, q, c);
      }
    }
    const double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[5] * J[6] - J[3] * J[8],
                 c02 = J[3] * J[7] - J[4] * J[6];
    const double det = J[0] * c00 + J[1] * c01 + J[2] * c02;
    if (!(det > 0.0)) ok = false;
    const double id = 1.0 / det;
    double Ji[9];
    Ji[0] = c00 * id; Ji[1] = (J[2] * J[7] - J[1] * J[8]) * id; Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
    Ji[3] = c01 * id; Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id; Ji[5] = (J[2] * J[3] - J[0] * J[5]) * id;
    Ji[6] = c02 * id; Ji[7] = (J[1] * J[6] - J[0] * J[7]) * id; Ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
    double A6[6];
    coef_at<3>(p, xq, tab, q, nfc, fc, A6);
    const double A[9] = {A6[0], A6[1], A6[2], A6[1], A6[3], A6[4], A6[2], A6[4], A6[5]};
    const double w = 0.125 * fabs(det);
    double G[8][3];  // physical gradients
    for (int k = 0; k < 8; ++k)
      for (int a = 0; a < 3; ++a) {
        double s = 0.0;
        for (int c = 0; c < 3; ++c) s += Ji[3 * c + a] * rgrad(k, q, c);
        G[k][a] = s;
      }
    for (int j = 0; j < 8; ++j) {
      double AG[3];
      for (int a = 0; a < 3; ++a) AG[a] = A[3 * a] * G[j][0] + A[3 * a + 1] * G[j][1] + A[3 * a + 2] * G[j][2];
      for (int i = 0; i <= j; ++i)
        K[tri_index(i, j)] += w * (G[i][0] * AG[0] + G[i][1] * AG[1] + G[i][2] * AG[2]);
    }
  }
  return ok;
}

// y = A~ v at node g for 8 RHS (SoA vectors with stride G).
template <typename T>
__device__ __forceinline__ void stencil27(const T *__restrict__ c, const T *__restrict__ v, long G,
                                          const int *offs, int g, T (&y)[8]) {
#pragma unroll
  for (int r = 0; r < 8; ++r) y[r] = v[r * G + g];
#pragma unroll 1
  for (int o = 0; o < 13; ++o) {
    const int d = offs[o];
    const T cf = c[o * G + g];
    const T cb = c[o * G + g - d];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      y[r] = fma(cf, v[r * G + g + d], y[r]);
      y[r] = fma(cb, v[r * G + g - d], y[r]);
    }
  }
}

// Node-major FP32 vectors ([node][8 RHS], 32-byte aligned nodes).
__device__ __forceinline__ void ld8(const float *__restrict__ v, int g, float (&t)[8]) {
  const float4 a = *reinterpret_cast<const float4 *>(v + 8 * (long)g);
  const float4 b = *reinterpret_cast<const float4 *>(v + 8 * (long)g + 4);
  t[0] = a.x; t[1] = a.y; t[2] = a.z; t[3] = a.w;
  t[4] = b.x; t[5] = b.y; t[6] = b.z; t[7] = b.w;
}
__device__ __forceinline__ void st8(float *__restrict__ v, int g, const float (&t)[8]) {
  *reinterpret_cast<float4 *>(v + 8 * (long)g) = make_float4(t[0], t[1], t[2], t[3]);
  *reinterpret_cast<float4 *>(v + 8 * (long)g + 4) = make_float4(t[4], t[5], t[6], t[7]);
}

// y = A~ v at node g for 8 RHS, v node-major; vc = v at g.  The same
// summation order as stencil27.
__device__ __forceinline__ void stencil27_nm(const float *__restrict__ c, const float *__restrict__ v, long G,
                                             const int *offs, int g, float (&y)[8], float (&vc)[8]) {
  ld8(v, g, vc);
#pragma unroll
  for (int r = 0; r < 8; ++r) y[r] = vc[r];
#pragma unroll
  for (int o = 0; o < 13; ++o) {
    const int d = offs[o];
    const float cf = c[o * G + g];
    const float cb = c[o * G + g - d];
    float tf[8], tb[8];
    ld8(v, g + d, tf);
    ld8(v, g - d, tb);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      y[r] = fmaf(cf, tf[r], y[r]);
      y[r] = fmaf(cb, tb[r], y[r]);
    }
  }
}

// Half H (RHS 4H .. 4H+3) of a node-major vector at node g: one 16-byte access.
template <int H>
__device__ __forceinline__ float4 ldh(const float *__restrict__ v, int g) {
  return *reinterpret_cast<const float4 *>(v + 8 * (long)g + 4 * H);
}
template <int H>
__device__ __forceinline__ void sth(float *__restrict__ v, int g, float4 t) {
  *reinterpret_cast<float4 *>(v + 8 * (long)g + 4 * H) = t;
}

// Index of the forward coupling (dx, dy, dz) among a node's 13 (compile-time
// offsets; the same order as fwd_offset / cs.offs).
__host__ __device__ constexpr int fwd_slot(int dx, int dy, int dz) {
  return dz == 1 ? 4 + (dy + 1) * 3 + (dx + 1) : (dy == 1 ? 1 + (dx + 1) : 0);
}
__host__ __device__ constexpr bool fwd_dir(int dx, int dy, int dz) {
  return dz > 0 || (dz == 0 && (dy > 0 || (dy == 0 && dx > 0)));
}

// Scaled coupling of node g with its neighbour at (dx, dy, dz) != 0: the
// node's own forward coupling, or the neighbour's forward coupling back.
template <int DX, int DY, int DZ>
__device__ __forceinline__ float coupling_nm(const float *__restrict__ c, long G, int P, int g) {
  if constexpr (fwd_dir(DX, DY, DZ)) return c[fwd_slot(DX, DY, DZ) * G + g];
  else return c[fwd_slot(-DX, -DY, -DZ) * G + g + (DZ * P + DY) * P + DX];
}

// q = A~ p for the z-pair of nodes g0 and g0 + P^2 (RHS 4H .. 4H+3 of the
// node-major p): the two 27-point stencils share 18 of their 36 neighbour
// sites, so the pair reads 36 sites instead of 54 (the inner loop is bound
// by L1 throughput).  Without a second node (two = false) y1, p1 stay 0.
template <int H, int SZ, int SY, int SX>
__device__ __forceinline__ void pair_site(const float *__restrict__ c, const float *__restrict__ v, long G,
                                          int P, int g0, bool two, float4 &y0, float4 &y1, float4 &p0,
                                          float4 &p1) {
  constexpr bool use0 = SZ <= 1;
  const bool use1 = two && SZ >= 0;
  const float4 t = (use0 || use1) ? ldh<H>(v, g0 + (SZ * P + SY) * P + SX) : make_float4(0.f, 0.f, 0.f, 0.f);
  if constexpr (use0) {
    if constexpr (SX == 0 && SY == 0 && SZ == 0) {
      p0 = t;
      y0.x += t.x; y0.y += t.y; y0.z += t.z; y0.w += t.w;
    } else {
      const float cf = coupling_nm<SX, SY, SZ>(c, G, P, g0);
      y0.x = fmaf(cf, t.x, y0.x); y0.y = fmaf(cf, t.y, y0.y);
      y0.z = fmaf(cf, t.z, y0.z); y0.w = fmaf(cf, t.w, y0.w);
    }
  }
  if constexpr (SZ >= 0) {
    if (use1) {
      if constexpr (SX == 0 && SY == 0 && SZ == 1) {
        p1 = t;
        y1.x += t.x; y1.y += t.y; y1.z += t.z; y1.w += t.w;
      } else {
        const float cf = coupling_nm<SX, SY, SZ - 1>(c, G, P, g0 + P * P);
        y1.x = fmaf(cf, t.x, y1.x); y1.y = fmaf(cf, t.y, y1.y);
        y1.z = fmaf(cf, t.z, y1.z); y1.w = fmaf(cf, t.w, y1.w);
      }
    }
  }
}
template <int H, int SZ, int SY>
__device__ __forceinline__ void pair_row(const float *__restrict__ c, const float *__restrict__ v, long G, int P,
                                         int g0, bool two, float4 &y0, float4 &y1, float4 &p0, float4 &p1) {
  pair_site<H, SZ, SY, -1>(c, v, G, P, g0, two, y0, y1, p0, p1);
  pair_site<H, SZ, SY, 0>(c, v, G, P, g0, two, y0, y1, p0, p1);
  pair_site<H, SZ, SY, 1>(c, v, G, P, g0, two, y0, y1, p0, p1);
}
template <int H, int SZ>
__device__ __forceinline__ void pair_plane(const float *__restrict__ c, const float *__restrict__ v, long G, int P,
                                           int g0, bool two, float4 &y0, float4 &y1, float4 &p0, float4 &p1) {
  pair_row<H, SZ, -1>(c, v, G, P, g0, two, y0, y1, p0, p1);
  asm volatile("" ::: "memory");
  pair_row<H, SZ, 0>(c, v, G, P, g0, two, y0, y1, p0, p1);
  asm volatile("" ::: "memory");
  pair_row<H, SZ, 1>(c, v, G, P, g0, two, y0, y1, p0, p1);
}
template <int H>
__device__ __forceinline__ void stencil27_pair(const float *__restrict__ c, const float *__restrict__ v, long G,
                                               int P, int g0, bool two, float4 &y0, float4 &y1, float4 &p0,
                                               float4 &p1) {
  y0 = y1 = p0 = p1 = make_float4(0.f, 0.f, 0.f, 0.f);
  // one row of sites' loads in flight at a time (the empty asm statements
  // keep the compiler from hoisting all 36 sites' loads, which would spill)
  pair_plane<H, -1>(c, v, G, P, g0, two, y0, y1, p0, p1);
  asm volatile("" ::: "memory");
  pair_plane<H, 0>(c, v, G, P, g0, two, y0, y1, p0, p1);
  asm volatile("" ::: "memory");
  pair_plane<H, 1>(c, v, G, P, g0, two, y0, y1, p0, p1);
  asm volatile("" ::: "memory");
  pair_plane<H, 2>(c, v, G, P, g0, two, y0, y1, p0, p1);
}

__device__ __forceinline__ int grid3(int P, int ix, int iy, int iz) { return ((iz + 1) * P + iy + 1) * P + ix + 1; }

// Geometry and Q1 data of one cell: corners, coupling offsets, BasisQ1
// coefficients, affine-cell Jacobian data and (scalar coefficients on affine
// cells) the per-Gauss-point element templates.  Sets cs.status.
template <int NT>
__device__ void cell_geometry3d(const KernelParams &p, CellShared3D &cs, int cell, int N, bool scalar,
                                int tid) {
  const int P = N + 3;
  if (tid < 24) cs.corners[tid] = p.corners[(int64_t)cell * 24 + tid];
  if (tid < 13) {
    int dx, dy, dz;
    fwd_offset(tid, dx, dy, dz);
    cs.offs[tid] = (dz * P + dy) * P + dx;
  }
  __syncthreads();
  if (tid == 0) {
    const double *cr = cs.corners;
    int st = MSFEM_CELL_CONVERGED;
    if (N < 1 || N > kNMax3D) st = MSFEM_CELL_BAD_INPUT;
    if (st == MSFEM_CELL_CONVERGED && !q1_setup<3>(cr, cs.q1coef, cs.q1shift, &cs.q1iscale))
      st = MSFEM_CELL_BAD_INPUT;
    // parallelepiped: v_k = v0 + kx e1 + ky e2 + kz e3 exactly
    int aff = 1;
    for (int k = 0; k < 8 && aff; ++k)
      for (int a = 0; a < 3; ++a) {
        const double pred = cr[a] + ((k & 1) ? cr[3 + a] - cr[a] : 0.0) + ((k & 2) ? cr[6 + a] - cr[a] : 0.0) +
                            ((k & 4) ? cr[12 + a] - cr[a] : 0.0);
        if (pred != cr[3 * k + a]) aff = 0;
      }
    cs.affine = aff;
    cs.refinements = 0;
    if (aff && st == MSFEM_CELL_CONVERGED) {
      const double invN = 1.0 / (double)N;
      double J[9];
      for (int a = 0; a < 3; ++a) {
        J[3 * a + 0] = (cr[3 + a] - cr[a]) * invN;
        J[3 * a + 1] = (cr[6 + a] - cr[a]) * invN;
        J[3 * a + 2] = (cr[12 + a] - cr[a]) * invN;
      }
      const double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[5] * J[6] - J[3] * J[8],
                   c02 = J[3] * J[7] - J[4] * J[6];
      const double det = J[0] * c00 + J[1] * c01 + J[2] * c02;
      if (!(det > 0.0)) st = MSFEM_CELL_BAD_INPUT;
      const double id = 1.0 / det;
      cs.jinv[0] = c00 * id; cs.jinv[1] = (J[2] * J[7] - J[1] * J[8]) * id; cs.jinv[2] = (J[1] * J[5] - J[2] * J[4]) * id;
      cs.jinv[3] = c01 * id; cs.jinv[4] = (J[0] * J[8] - J[2] * J[6]) * id; cs.jinv[5] = (J[2] * J[3] - J[0] * J[5]) * id;
      cs.jinv[6] = c02 * id; cs.jinv[7] = (J[1] * J[6] - J[0] * J[7]) * id; cs.jinv[8] = (J[0] * J[4] - J[1] * J[3]) * id;
      for (int e = 0; e < 9; ++e) cs.jfine[e] = J[e];
      cs.absdet = fabs(det);
    }
    cs.status = st;
  }
  __syncthreads();
  // element templates for a scalar coefficient on an affine cell:
  // tmpl[q](i,j) = w|det| (Ji^T grad_i) . (Ji^T grad_j) at Gauss point q
  if (cs.status == MSFEM_CELL_CONVERGED && cs.affine && scalar) {
    for (int e = tid; e < 8 * 36; e += NT) {
      const int q = e / 36, t = e % 36;
      int i = 0, rem = t;
      while (rem >= 8 - i) { rem -= 8 - i; ++i; }
      const int j = i + rem;
      double gi[3], gj[3];
      for (int a = 0; a < 3; ++a) {
        double si = 0.0, sj = 0.0;
        for (int c = 0; c < 3; ++c) {
          si += cs.jinv[3 * c + a] * rgrad(i, q, c);
          sj += cs.jinv[3 * c + a] * rgrad(j, q, c);
        }
        gi[a] = si;
        gj[a] = sj;
      }
      cs.tmpl[q][t] = 0.125 * cs.absdet * (gi[0] * gj[0] + gi[1] * gj[1] + gi[2] * gj[2]);
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Thread-block clusters: CS CTAs share one cell (CS = 1: one CTA per cell).
// The cluster's CTAs split every node loop, meet at cluster barriers (release /
// acquire at cluster scope, so workspace writes before a barrier are seen
// after it), and sum reduction partials read from each other's shared memory
// in a fixed rank order, so all CTAs take the same decisions.
// ---------------------------------------------------------------------------
template <int CS>
__device__ __forceinline__ int cluster_rank() {
  if constexpr (CS > 1) return (int)cooperative_groups::this_cluster().block_rank();
  else return 0;
}
template <int CS>
__device__ __forceinline__ void csync() {
  if constexpr (CS > 1) cooperative_groups::this_cluster().sync();
  else __syncthreads();
}
// The same shared-memory object in CTA `rank` of the cluster.
template <int CS, typename T>
__device__ __forceinline__ T *peer(T *ptr, int rank) {
  if constexpr (CS > 1) return cooperative_groups::this_cluster().map_shared_rank(ptr, rank);
  else return ptr;
}

// One refinement segment of the mixed form's inner FP32 CG (at most
// inner_maxit iterations, per-RHS stopping at r.r <= thr) on the node-major
// FP32 vectors.  Kept out of line: the kernel's FP64-phase state is saved
// once per segment rather than held in registers through the FP32 loop (the
// 2-CTA/SM shapes run at 64 registers per thread).  Reductions use red[buf],
// red[buf ^ 1] alternately, buf as left by the caller's last reduction.
template <int NT, int CS, int PC>
__device__ __noinline__ void inner_segment3d(const float *__restrict__ c32, float *pp32, float *qq32,
                                             float *rr32, float *dd32, long G, int m, int P, int nI,
                                             int inner_maxit, unsigned iact, int buf,
                                             double (*red)[NT / 32 * 16], CellShared3D &cs) {
  constexpr int NW = NT / 32;
  constexpr int CNT = NT * CS;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ctid = cluster_rank<CS>() * NT + tid;
  auto interior = [&](int k) {
    if constexpr (PC > 0) {
      // compile-time m and P: the divisions become multiplications
      constexpr int mc = PC - 4;
      const int ix = 1 + k % mc, iy = 1 + (k / mc) % mc, iz = 1 + k / (mc * mc);
      return grid3(PC, ix, iy, iz);
    } else {
      const int ix = 1 + k % m, iy = 1 + (k / m) % m, iz = 1 + k / (m * m);
      return grid3(P, ix, iy, iz);
    }
  };

  auto block_sum8 = [&](float (&v)[8]) {
    float vv[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) vv[r] = v[r];
    const float t = warp_transpose_reduce<8>(vv, lane);
    float *rb = reinterpret_cast<float *>(red[buf]);
    if ((lane & 3) == 0) rb[warp * 8 + (lane >> 2)] = t;
    csync<CS>();
    float s = 0.f;
    for (int c = 0; c < CS; ++c) {
      const float *rc = peer<CS>(rb, c);
      for (int i = lane; i < NW * 8; i += 32) s += rc[i];
    }
#pragma unroll
    for (int mm = 8; mm < 32; mm <<= 1) s += shfl_xor_d(s, mm);
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = __shfl_sync(0xffffffffu, s, r);
    buf ^= 1;
  };
  // r.r per RHS in shared memory (seg_rho[par], double-buffered so that
  // every thread reads the old values while the next ones are written) and
  // the stopping thresholds seg_thr: 16 registers fewer in the node loops
  int par = 0;
  int iit = 0;
  for (;;) {
    if (!iact || iit >= inner_maxit) break;
    ++iit;
    float sg[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) sg[r] = 0.f;
    if constexpr (PC == 0) {
      // any N: one node (8 RHS) per thread
      for (int k = ctid; k < nI; k += CNT) {
        const int g = interior(k);
        float y[8], pc[8];
        stencil27_nm(c32, pp32, G, cs.offs, g, y, pc);
        st8(qq32, g, y);
#pragma unroll
        for (int r = 0; r < 8; ++r) sg[r] = fmaf(pc[r], y[r], sg[r]);
      }
    } else {
    // q = A~ p and p.q over z-pairs of interior nodes (iz, iz + 1), iz odd;
    // with m odd the last layer holds single nodes.  P = PC is a compile-
    // time constant here, so the 36 site offsets are immediates.
    constexpr int P = PC, m = PC - 4, mz = (m + 1) / 2;
    constexpr long GC = (long)PC * PC * PC;  // = G: coupling offsets are immediates too
    for (int k = ctid; k < m * m * mz; k += CNT) {
      const int ix = 1 + k % m, iy = 1 + (k / m) % m, iz = 1 + 2 * (k / (m * m));
      const bool two = iz < m;
      const int g0 = grid3(P, ix, iy, iz);
      float4 y0, y1, p0, p1;
      stencil27_pair<0>(c32, pp32, GC, P, g0, two, y0, y1, p0, p1);
      sth<0>(qq32, g0, y0);
      if (two) sth<0>(qq32, g0 + P * P, y1);
      sg[0] = fmaf(p0.x, y0.x, fmaf(p1.x, y1.x, sg[0]));
      sg[1] = fmaf(p0.y, y0.y, fmaf(p1.y, y1.y, sg[1]));
      sg[2] = fmaf(p0.z, y0.z, fmaf(p1.z, y1.z, sg[2]));
      sg[3] = fmaf(p0.w, y0.w, fmaf(p1.w, y1.w, sg[3]));
      stencil27_pair<1>(c32, pp32, GC, P, g0, two, y0, y1, p0, p1);
      sth<1>(qq32, g0, y0);
      if (two) sth<1>(qq32, g0 + P * P, y1);
      sg[4] = fmaf(p0.x, y0.x, fmaf(p1.x, y1.x, sg[4]));
      sg[5] = fmaf(p0.y, y0.y, fmaf(p1.y, y1.y, sg[5]));
      sg[6] = fmaf(p0.z, y0.z, fmaf(p1.z, y1.z, sg[6]));
      sg[7] = fmaf(p0.w, y0.w, fmaf(p1.w, y1.w, sg[7]));
    }
    }
    block_sum8(sg);
    float al[8], rp[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      al[r] = (((iact >> r) & 1u) && sg[r] > 0.f) ? cs.seg_rho[par][r] / sg[r] : 0.0f;
      rp[r] = 0.f;
    }
    for (int k = ctid; k < nI; k += CNT) {
      const int g = interior(k);
      float dv[8], pv[8], qv[8], rv[8];
      ld8(dd32, g, dv);
      ld8(pp32, g, pv);
      ld8(qq32, g, qv);
      ld8(rr32, g, rv);
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        dv[r] = fmaf(al[r], pv[r], dv[r]);
        rv[r] = fmaf(-al[r], qv[r], rv[r]);
        rp[r] = fmaf(rv[r], rv[r], rp[r]);
      }
      st8(dd32, g, dv);
      st8(rr32, g, rv);
    }
    block_sum8(rp);
    float be[8];
    if (tid < 8 && ((iact >> tid) & 1u)) cs.inner_iters[tid] += 1;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      be[r] = 0.0f;
      const float rho = cs.seg_rho[par][r];
      float next = rho;
      if ((iact >> r) & 1u) {
        if (!(rp[r] <= cs.seg_thr[r]) && isfinite(rp[r])) {
          be[r] = rp[r] / rho;
          next = rp[r];
        } else {
          iact &= ~(1u << r);
        }
      }
      if (tid == r) cs.seg_rho[par ^ 1][r] = next;
    }
    par ^= 1;
    for (int k = ctid; k < nI; k += CNT) {
      const int g = interior(k);
      float pv[8], rv[8];
      ld8(pp32, g, pv);
      ld8(rr32, g, rv);
#pragma unroll
      for (int r = 0; r < 8; ++r) pv[r] = fmaf(be[r], pv[r], rv[r]);
      st8(pp32, g, pv);
    }
    csync<CS>();
  }
}

// ---------------------------------------------------------------------------
// On-chip inner loop of the cluster shape (mixed form).  The CS CTAs of a
// cluster split the cell's interior z-planes into contiguous slabs of at most
// SMAX planes (block partition, empty slabs last).  Each CTA keeps in shared
// memory
//   - the inner residual r of its planes plus one halo plane on either side
//     (RHS 0-3 and 4-7 in two float4 arrays, so a warp's 16-byte loads hit
//     distinct banks), in planes of fixed row stride kRS and plane stride kPS
//     whose last column and row stay zero: the cell's zero Dirichlet ring,
//     reached at compile-time offsets without bounds tests;
//   - the FP32 couplings of its planes (13 forward ones per interior node,
//     row stride kMaxM) plus the 9 upward couplings of the plane below;
//   - RHS 4-7 of the correction d of its nodes.
// A thread owns one (x, y) column of the slab; its search direction p, A p
// and RHS 0-3 of d stay in registers.  The CG runs in the form that applies
// the stencil to r: q = A r + beta q equals A p for p = r + beta p, so one
// cluster barrier covers both the halo exchange of r and the sum of r.r, and
// the other the sum of p.q: two cluster barriers per iteration.  Global
// memory is read once per segment (r, couplings) and written once (d).
// ---------------------------------------------------------------------------
template <int SMAX>
struct Slab3D {
  static constexpr int kMaxM = kNMax3D - 1;          // interior nodes per direction
  static constexpr int kRS = kMaxM + 1;              // row stride of the r planes (one zero column)
  static constexpr int kPS = kRS * (kMaxM + 1);      // plane stride of the r planes (one zero row)
  static constexpr int kPad = 32;                    // zero entries before the first r plane
  static constexpr int kMaxCol = kMaxM * kMaxM;      // coupling plane (row stride kMaxM)
  static constexpr int kCPad = 32;                   // zero couplings before and after
  static constexpr size_t kV = size_t(kPad + (SMAX + 2) * kPS) * 16;                 // one half of r
  static constexpr size_t kCpl = size_t(2 * kCPad + (SMAX * 13 + 9) * kMaxCol) * 4;
  static constexpr size_t kD = size_t(SMAX) * kMaxCol * 16;                          // RHS 4-7 of d
  static constexpr size_t kPart = 2 * 8 * 4;                                         // cluster-sum partials
  static constexpr size_t bytes = 2 * kV + kCpl + kD + kPart;
  static_assert(kV % 16 == 0 && kCpl % 16 == 0 && kD % 16 == 0, "16-byte aligned regions");
};

// Slab of cluster rank c: planes [lo, lo + S) of the m interior planes.
__device__ __forceinline__ void slab_range(int m, int CS, int c, int &lo, int &S) {
  const int base = m / CS, extra = m % CS;
  lo = 1 + c * base + min(c, extra);
  S = c < CS ? base + (c < extra ? 1 : 0) : 0;
}

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// One xy-site (DX, DY) of a column's stencil: the r values of the site in
// every plane of the slab and its halos, applied to every owned node within
// one plane of it.  A node's coupling with the site is its own forward
// coupling, or the neighbour's forward coupling back (for the plane below the
// slab, from the halo coupling block).  At a site on the cell's boundary r is
// zero, so whatever finite coupling the compile-time offset reads there
// contributes nothing.
template <int SMAX, int DX, int DY>
__device__ __forceinline__ void slab_site(const float4 *__restrict__ rlo, const float4 *__restrict__ rhi,
                                          const float *__restrict__ cpl, int lpos, int ccol, int S,
                                          float2 (&q)[SMAX][4]) {
  using S3 = Slab3D<SMAX>;
  constexpr int kRoff = DY * S3::kRS + DX, kCoff = DY * S3::kMaxM + DX;
#pragma unroll
  for (int zz = 0; zz < SMAX + 2; ++zz) {
    if (zz >= S + 2) break;
    const float4 a = rlo[zz * S3::kPS + lpos + kRoff];
    const float4 b = rhi[zz * S3::kPS + lpos + kRoff];
#pragma unroll
    for (int s = 0; s < SMAX; ++s) {
      const int dz = zz - 1 - s;
      if (dz < -1 || dz > 1 || s >= S) continue;
      float c;
      if (DX == 0 && DY == 0 && dz == 0) {
        c = 1.0f;  // the scaled operator has a unit diagonal
      } else if (fwd_dir(DX, DY, dz)) {
        c = cpl[(s * 13 + fwd_slot(DX, DY, dz)) * S3::kMaxCol + ccol];
      } else if (dz == 0) {
        c = cpl[(s * 13 + fwd_slot(-DX, -DY, 0)) * S3::kMaxCol + ccol + kCoff];
      } else if (s >= 1) {
        c = cpl[((s - 1) * 13 + fwd_slot(-DX, -DY, 1)) * S3::kMaxCol + ccol + kCoff];
      } else {
        c = cpl[(SMAX * 13 + fwd_slot(-DX, -DY, 1) - 4) * S3::kMaxCol + ccol + kCoff];
      }
      const float2 cc = f2(c, c);
      q[s][0] = __ffma2_rn(cc, f2(a.x, a.y), q[s][0]);
      q[s][1] = __ffma2_rn(cc, f2(a.z, a.w), q[s][1]);
      q[s][2] = __ffma2_rn(cc, f2(b.x, b.y), q[s][2]);
      q[s][3] = __ffma2_rn(cc, f2(b.z, b.w), q[s][3]);
    }
  }
}

template <int SMAX, int DY>
__device__ __forceinline__ void slab_row(const float4 *__restrict__ rlo, const float4 *__restrict__ rhi,
                                         const float *__restrict__ cpl, int lpos, int ccol, int S,
                                         float2 (&q)[SMAX][4]) {
  slab_site<SMAX, -1, DY>(rlo, rhi, cpl, lpos, ccol, S, q);
  slab_site<SMAX, 0, DY>(rlo, rhi, cpl, lpos, ccol, S, q);
  slab_site<SMAX, 1, DY>(rlo, rhi, cpl, lpos, ccol, S, q);
}

// Sum of 8 values over every thread of the cluster, in a fixed order (warp
// transposes, the CTA's warps in order, then the CTAs in rank order with a
// commutative butterfly), so every thread of every CTA gets the same bits.
// Includes the cluster barrier that publishes the shared-memory writes made
// before the call (the partials, and the halo planes pushed to neighbours).
template <int NT, int CS>
__device__ __forceinline__ void cluster_sum8(float (&v)[8], float *redw, float *part, int slot, int lane,
                                             int warp) {
  constexpr int NW = NT / 32;
  float vv[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) vv[r] = v[r];
  const float t = warp_transpose_reduce<8>(vv, lane);
  if ((lane & 3) == 0) redw[warp * 8 + (lane >> 2)] = t;
  __syncthreads();
  if (warp == 0 && lane < 8) {
    float s = 0.f;
    for (int w = 0; w < NW; ++w) s += redw[w * 8 + lane];
    part[slot * 8 + lane] = s;
  }
  csync<CS>();
  float s = 0.f;
  for (int c = lane >> 3; c < CS; c += 4) s += peer<CS>(part, c)[slot * 8 + (lane & 7)];
  s += shfl_xor_d(s, 8);
  s += shfl_xor_d(s, 16);
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = __shfl_sync(0xffffffffu, s, r);
}

// One refinement segment of the inner FP32 CG on the slabs (see above).
// In: rr32 = the FP32 residual on every interior node (node-major), written
// before the last cluster barrier; cs.seg_rho[0] = r.r, cs.seg_thr the
// stopping thresholds.  Out: dd32 = the correction on every interior node,
// visible to the whole cluster on return.
template <int NT, int CS, int SMAX>
__device__ __noinline__ void inner_segment3d_slab(const float *__restrict__ c32, const float *__restrict__ rr32,
                                                  float *__restrict__ dd32, long G, int N, int P, int inner_maxit,
                                                  unsigned iact, float *redw, CellShared3D &cs,
                                                  unsigned char *dsm) {
  using S3 = Slab3D<SMAX>;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int crank = cluster_rank<CS>();
  const int m = N - 1, mm = m * m;
  int lo, S, lo_nb, S_dn, S_up;
  slab_range(m, CS, crank, lo, S);
  slab_range(m, CS, crank > 0 ? crank - 1 : 0, lo_nb, S_dn);
  slab_range(m, CS, crank + 1, lo_nb, S_up);
  float4 *rlo = reinterpret_cast<float4 *>(dsm) + S3::kPad;
  float4 *rhi = reinterpret_cast<float4 *>(dsm + S3::kV) + S3::kPad;
  float *cpl = reinterpret_cast<float *>(dsm + 2 * S3::kV) + S3::kCPad;
  float4 *dhi = reinterpret_cast<float4 *>(dsm + 2 * S3::kV + S3::kCpl);
  float *part = reinterpret_cast<float *>(dsm + 2 * S3::kV + S3::kCpl + S3::kD);
  const bool own = tid < mm && S > 0;
  const int col = own ? tid : 0;
  const int ix = 1 + col % m, iy = 1 + col / m;
  const int lpos = (iy - 1) * S3::kRS + (ix - 1);     // position in an r plane
  const int ccol = (iy - 1) * S3::kMaxM + (ix - 1);   // position in a coupling plane
  const int rdn = crank > 0 ? crank - 1 : crank, rup = crank + 1 < CS ? crank + 1 : crank;
  const bool push_dn = own && crank > 0;
  const bool push_up = own && crank + 1 < CS && S_up > 0;

  // set-up: zero r (halo planes on the cell's boundary, the zero ring) and the
  // couplings (padding, unused positions), then load this slab's couplings
  {
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 *v = reinterpret_cast<float4 *>(dsm);
    for (int i = tid; i < (int)(2 * S3::kV / 16); i += NT) v[i] = z4;
    float *c = reinterpret_cast<float *>(dsm + 2 * S3::kV);
    for (int i = tid; i < (int)(S3::kCpl / 4); i += NT) c[i] = 0.f;
  }
  __syncthreads();
  for (int i = tid; i < S * 13 * mm; i += NT) {
    const int c = i % mm, so = i / mm, o = so % 13, sl = so / 13;
    const int jx = c % m, jy = c / m;
    cpl[(sl * 13 + o) * S3::kMaxCol + jy * S3::kMaxM + jx] = c32[o * G + grid3(P, 1 + jx, 1 + jy, lo + sl)];
  }
  if (lo - 1 >= 1)
    for (int i = tid; i < 9 * mm; i += NT) {
      const int c = i % mm, j = i / mm;
      const int jx = c % m, jy = c / m;
      cpl[(SMAX * 13 + j) * S3::kMaxCol + jy * S3::kMaxM + jx] = c32[(4 + j) * G + grid3(P, 1 + jx, 1 + jy, lo - 1)];
    }
  csync<CS>();  // every CTA's r is zeroed before any halo is pushed into it
  // the neighbours' addresses are mapped at each push (few registers live
  // through the inner loop: the 17-warp shape runs at 96 per thread)
  auto push_halos = [&]() {
    if (push_dn) {  // bottom plane -> the top halo of the CTA below
      peer<CS>(rlo, rdn)[(S_dn + 1) * S3::kPS + lpos] = rlo[S3::kPS + lpos];
      peer<CS>(rhi, rdn)[(S_dn + 1) * S3::kPS + lpos] = rhi[S3::kPS + lpos];
    }
    if (push_up) {  // top plane -> the bottom halo of the CTA above
      peer<CS>(rlo, rup)[lpos] = rlo[S * S3::kPS + lpos];
      peer<CS>(rhi, rup)[lpos] = rhi[S * S3::kPS + lpos];
    }
  };
  float2 p[SMAX][4], q[SMAX][4], dlo[SMAX][2];
#pragma unroll
  for (int sl = 0; sl < SMAX; ++sl) {
    if (own && sl < S) {
      float t[8];
      ld8(rr32, grid3(P, ix, iy, lo + sl), t);
      rlo[(sl + 1) * S3::kPS + lpos] = make_float4(t[0], t[1], t[2], t[3]);
      rhi[(sl + 1) * S3::kPS + lpos] = make_float4(t[4], t[5], t[6], t[7]);
      dhi[sl * S3::kMaxCol + ccol] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) p[sl][k] = q[sl][k] = f2(0.f, 0.f);
    dlo[sl][0] = dlo[sl][1] = f2(0.f, 0.f);
  }
  if (tid < 8) cs.seg_beta[tid] = 0.0f;  // 0: p = r, q = A r on the first pass
  push_halos();
  csync<CS>();

  int par = 0;
  for (int iit = 0; iit < inner_maxit && iact; ++iit) {
    // q = A~ r + beta q, p = r + beta p on the owned column; p.q
#pragma unroll
    for (int sl = 0; sl < SMAX; ++sl)
#pragma unroll
      for (int k = 0; k < 4; ++k)
        q[sl][k] = __fmul2_rn(f2(cs.seg_beta[2 * k], cs.seg_beta[2 * k + 1]), q[sl][k]);
    if (own) {
      slab_row<SMAX, -1>(rlo, rhi, cpl, lpos, ccol, S, q);
      slab_row<SMAX, 0>(rlo, rhi, cpl, lpos, ccol, S, q);
      slab_row<SMAX, 1>(rlo, rhi, cpl, lpos, ccol, S, q);
    }
    float2 sg2[4] = {f2(0.f, 0.f), f2(0.f, 0.f), f2(0.f, 0.f), f2(0.f, 0.f)};
#pragma unroll
    for (int sl = 0; sl < SMAX; ++sl) {
      if (own && sl < S) {
        const float4 a = rlo[(sl + 1) * S3::kPS + lpos], b = rhi[(sl + 1) * S3::kPS + lpos];
        const float2 rv[4] = {f2(a.x, a.y), f2(a.z, a.w), f2(b.x, b.y), f2(b.z, b.w)};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          p[sl][k] = __ffma2_rn(f2(cs.seg_beta[2 * k], cs.seg_beta[2 * k + 1]), p[sl][k], rv[k]);
          sg2[k] = __ffma2_rn(p[sl][k], q[sl][k], sg2[k]);
        }
      }
    }
    float sg[8] = {sg2[0].x, sg2[0].y, sg2[1].x, sg2[1].y, sg2[2].x, sg2[2].y, sg2[3].x, sg2[3].y};
    cluster_sum8<NT, CS>(sg, redw, part, 0, lane, warp);
    float al[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) al[k] = (((iact >> k) & 1u) && sg[k] > 0.f) ? cs.seg_rho[par][k] / sg[k] : 0.0f;
    // d += alpha p, r -= alpha q (r in shared memory, pushed to the halos), r.r
    float2 rp2[4] = {f2(0.f, 0.f), f2(0.f, 0.f), f2(0.f, 0.f), f2(0.f, 0.f)};
#pragma unroll
    for (int sl = 0; sl < SMAX; ++sl) {
      if (own && sl < S) {
        const int pi = (sl + 1) * S3::kPS + lpos;
        const float4 a = rlo[pi], b = rhi[pi];
        float2 rv[4] = {f2(a.x, a.y), f2(a.z, a.w), f2(b.x, b.y), f2(b.z, b.w)};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          rv[k] = __ffma2_rn(f2(-al[2 * k], -al[2 * k + 1]), q[sl][k], rv[k]);
          rp2[k] = __ffma2_rn(rv[k], rv[k], rp2[k]);
        }
        rlo[pi] = make_float4(rv[0].x, rv[0].y, rv[1].x, rv[1].y);
        rhi[pi] = make_float4(rv[2].x, rv[2].y, rv[3].x, rv[3].y);
        dlo[sl][0] = __ffma2_rn(f2(al[0], al[1]), p[sl][0], dlo[sl][0]);
        dlo[sl][1] = __ffma2_rn(f2(al[2], al[3]), p[sl][1], dlo[sl][1]);
        float4 dh = dhi[sl * S3::kMaxCol + ccol];
        const float2 d45 = __ffma2_rn(f2(al[4], al[5]), p[sl][2], f2(dh.x, dh.y));
        const float2 d67 = __ffma2_rn(f2(al[6], al[7]), p[sl][3], f2(dh.z, dh.w));
        dhi[sl * S3::kMaxCol + ccol] = make_float4(d45.x, d45.y, d67.x, d67.y);
      }
    }
    push_halos();
    float rp[8] = {rp2[0].x, rp2[0].y, rp2[1].x, rp2[1].y, rp2[2].x, rp2[2].y, rp2[3].x, rp2[3].y};
    cluster_sum8<NT, CS>(rp, redw, part, 1, lane, warp);
    if (tid < 8 && ((iact >> tid) & 1u)) cs.inner_iters[tid] += 1;
    // beta and the next r.r by thread k; every thread updates the active set.
    // The barrier below orders these writes before the next iteration's reads
    // (and the reads of seg_rho[par] above before the next writes to it).
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float be = 0.0f;
      const float rho = cs.seg_rho[par][k];
      float next = rho;
      if ((iact >> k) & 1u) {
        if (!(rp[k] <= cs.seg_thr[k]) && isfinite(rp[k])) {
          be = rp[k] / rho;
          next = rp[k];
        } else {
          iact &= ~(1u << k);
        }
      }
      if (tid == k) {
        cs.seg_rho[par ^ 1][k] = next;
        cs.seg_beta[k] = be;
      }
    }
    par ^= 1;
    __syncthreads();
  }
  // the correction of the owned nodes, for the FP64 update of the whole cluster
#pragma unroll
  for (int sl = 0; sl < SMAX; ++sl)
    if (own && sl < S) {
      const float4 dh = dhi[sl * S3::kMaxCol + ccol];
      const float dv[8] = {dlo[sl][0].x, dlo[sl][0].y, dlo[sl][1].x, dlo[sl][1].y, dh.x, dh.y, dh.z, dh.w};
      st8(dd32, grid3(P, ix, iy, lo + sl), dv);
    }
  csync<CS>();
}

template <int NT, bool MIXED, int MINB, int CS>
__global__ void __launch_bounds__(NT, MINB)
msfem3d_kernel(const KernelParams p, unsigned char *__restrict__ work, size_t slot_bytes) {
  constexpr int NW = NT / 32;
  constexpr int CNT = NT * CS;  // threads working on one cell (the cluster's)
  __shared__ CellShared3D cs;
  __shared__ double red[2][NW * 16];
  // the slab cluster shape reuses its dynamic shared memory (idle in the
  // epilogue) for the epilogue partials
  constexpr bool kSlab = MIXED && CS > 1;
  __shared__ double redE_static[kSlab ? 1 : NW * 32];
  extern __shared__ __align__(16) unsigned char dsm3[];
  double *redE = kSlab ? reinterpret_cast<double *>(dsm3) : redE_static;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int crank = cluster_rank<CS>();  // this CTA's rank in its cluster
  const int ctid = crank * NT + tid;     // thread index within the cluster
  // one workspace slot per cluster
  unsigned char *slot = work + (size_t)(blockIdx.x / CS) * slot_bytes;
  // every CTA of the cluster ends with the same cell status (the first
  // non-converged one in rank order)
  auto agree_status = [&]() {
    if constexpr (CS > 1) {
      csync<CS>();
      int st = MSFEM_CELL_CONVERGED;
      if (tid == 0)
        for (int c = 0; c < CS; ++c) {
          const int s2 = *peer<CS>(&cs.status, c);
          if (st == MSFEM_CELL_CONVERGED) st = s2;
        }
      csync<CS>();
      if (tid == 0) cs.status = st;
      __syncthreads();
    }
  };
  double *W64 = reinterpret_cast<double *>(slot);
  float *W32 = reinterpret_cast<float *>(slot + sizeof(double) * Work3D::kEnd64);

  for (;;) {
    if (tid == 0 && crank == 0) {
      const unsigned wi = atomicAdd(p.queue, 1u);
      cs.cell = wi < (unsigned)p.n_cells ? (p.order ? p.order[wi] : (int)wi) : -1;
    }
    csync<CS>();
    const int cell = *peer<CS>(&cs.cell, 0);
    if constexpr (CS > 1) csync<CS>();  // rank 0's shared memory is read before any CTA may exit
    if (cell < 0) break;
    const int N = p.n_fine ? p.n_fine[cell] : p.n_fine_uniform;
    const int P = N + 3, n = N + 1, m = N - 1;
    const long G = (long)P * P * P;
    const int nI = m * m * m, nn = n * n * n;
    double *c64 = W64 + Work3D::kC64 * 0 + 0;  // strides use this cell's G
    double *d64 = c64 + 13 * G;
    double *x64 = d64 + G;
    double *r64 = x64 + 8 * G;
    double *p64 = r64 + 8 * G;
    double *q64 = p64 + 8 * G;
    // this cell's layout of the same slot (G <= Work3D::G, so G4 <= Work3D::G4)
    const long G4 = (G + 3) & ~3L;
    float *c32 = W32;
    float *dd32 = c32 + 13 * G4;  // 16-byte aligned: node-major float4 accesses
    float *rr32 = dd32 + 8 * G4;
    float *pp32 = rr32 + 8 * G4;
    float *qq32 = pp32 + 8 * G4;

    // ---------------- set-up ------------------------------------------
    if (tid < 8) { cs.iters[tid] = 0; cs.active[tid] = 1; cs.nu[tid] = 0.0; }
    for (long i = ctid; i < 22 * G; i += CNT) c64[i] = 0.0;  // couplings, diagonal, phi~
    const bool scalar = (p.coef_kind == MSFEM_COEF_TABULATED && p.ncomp == 1) ||
                        p.coef_kind == MSFEM_COEF_SINSIN;
    cell_geometry3d<NT>(p, cs, cell, N, scalar, tid);
    if (cs.status != MSFEM_CELL_CONVERGED) {
      if (crank == 0) {
        for (int i = tid; i < 64; i += NT) p.M[(int64_t)cell * 64 + i] = __longlong_as_double(0x7ff8000000000000ll);
        if (tid < 8) {
          p.F[(int64_t)cell * 8 + tid] = __longlong_as_double(0x7ff8000000000000ll);
          if (p.iters) p.iters[(int64_t)cell * 8 + tid] = 0;
        }
        if (tid == 0) {
          p.status[cell] = cs.status;
          if (p.rel_res) p.rel_res[cell] = __longlong_as_double(0x7ff8000000000000ll);
          if (p.refinements) p.refinements[cell] = 0;
        }
      }
      csync<CS>();
      continue;
    }

    csync<CS>();  // the workspace is zeroed by all CTAs of the cluster
    // ---------------- assembly: 8-colour scatter -------------------------
    {
      const int nfc = N * N * N;
      const double *tab = nullptr;
      if (p.coef_kind == MSFEM_COEF_TABULATED)
        tab = p.qp_values + (p.qp_offset ? p.qp_offset[cell] : (int64_t)cell * p.ncomp * 8 * nfc);
      const bool need_x = p.coef_kind != MSFEM_COEF_TABULATED && p.coef_kind != MSFEM_COEF_CONSTANT;
      for (int col = 0; col < 8; ++col) {
        const int ox = col & 1, oy = (col >> 1) & 1, oz = col >> 2;
        const int nx = (N - ox + 1) >> 1, ny = (N - oy + 1) >> 1, nz = (N - oz + 1) >> 1;
        for (int idx = ctid; idx < nx * ny * nz; idx += CNT) {
          const int cx = ox + 2 * (idx % nx), cy = oy + 2 * ((idx / nx) % ny), cz = oz + 2 * (idx / (nx * ny));
          double K[36];
          if (!element3d(p, cs, tab, N, cx, cy, cz, scalar, need_x, K)) cs.status = MSFEM_CELL_BAD_INPUT;
          const int g0 = grid3(P, cx, cy, cz);
#pragma unroll 1
          for (int i = 0; i < 8; ++i) {
            const int gi = g0 + ((i >> 2) * P + ((i >> 1) & 1)) * P + (i & 1);
            d64[gi] += K[tri_index(i, i)];
            for (int j = i + 1; j < 8; ++j) {
              int dx = (j & 1) - (i & 1), dy = ((j >> 1) & 1) - ((i >> 1) & 1), dz = (j >> 2) - (i >> 2);
              int base = gi;
              if (!is_forward(dx, dy, dz)) {
                base = gi + (dz * P + dy) * P + dx;
                dx = -dx; dy = -dy; dz = -dz;
              }
              c64[(long)fwd_index(dx, dy, dz) * G + base] += K[tri_index(i, j)];
            }
          }
        }
        csync<CS>();
      }
    }
    agree_status();
    if (cs.status != MSFEM_CELL_CONVERGED) {
      if (crank == 0) {
        for (int i = tid; i < 64; i += NT) p.M[(int64_t)cell * 64 + i] = __longlong_as_double(0x7ff8000000000000ll);
        if (tid < 8) {
          p.F[(int64_t)cell * 8 + tid] = __longlong_as_double(0x7ff8000000000000ll);
          if (p.iters) p.iters[(int64_t)cell * 8 + tid] = 0;
        }
        if (tid == 0) {
          p.status[cell] = cs.status;
          if (p.rel_res) p.rel_res[cell] = __longlong_as_double(0x7ff8000000000000ll);
          if (p.refinements) p.refinements[cell] = 0;
        }
      }
      csync<CS>();
      continue;
    }

    // ---------------- symmetric scaling, Dirichlet data --------------------
    // D^-1/2 temporarily in r64[0]
    double dmin_part = 1e300;
    for (int k = ctid; k < nn; k += CNT) {
      const int ix = k % n, iy = (k / n) % n, iz = k / (n * n);
      const int g = grid3(P, ix, iy, iz);
      const double d = d64[g];
      r64[g] = rsqrt(d);
      if (ix > 0 && iy > 0 && iz > 0 && ix < N && iy < N && iz < N) {
        dmin_part = fmin(dmin_part, d);
        if (!(d > 0.0) || !isfinite(d)) cs.status = MSFEM_CELL_NAN;
      }
    }
    // zero the ring entries of the temporary (read by the scaling below)
    for (long i = ctid; i < G; i += CNT) {
      const int ix = (int)(i % P) - 1, iy = (int)((i / P) % P) - 1, iz = (int)(i / ((long)P * P)) - 1;
      if (ix < 0 || iy < 0 || iz < 0 || ix > N || iy > N || iz > N) r64[i] = 0.0;
    }
    csync<CS>();
    for (int k = ctid; k < nn; k += CNT) {
      const int ix = k % n, iy = (k / n) % n, iz = k / (n * n);
      const int g = grid3(P, ix, iy, iz);
      const double s = r64[g];
#pragma unroll 1
      for (int o = 0; o < 13; ++o) c64[o * G + g] *= s * r64[g + cs.offs[o]];
    }
#pragma unroll
    for (int mm = 16; mm >= 1; mm >>= 1) dmin_part = fmin(dmin_part, shfl_xor_d(dmin_part, mm));
    if (lane == 0) red[0][warp] = dmin_part;
    csync<CS>();
    for (int k = ctid; k < nn; k += CNT) {
      const int ix = k % n, iy = (k / n) % n, iz = k / (n * n);
      const int g = grid3(P, ix, iy, iz);
      if (ix == 0 || iy == 0 || iz == 0 || ix == N || iy == N || iz == N) {
        const double t[3] = {ix / (double)N, iy / (double)N, iz / (double)N};
        double x[3], gv[8];
        trilinear_map(cs.corners, t, x);
        q1_eval<3>(cs.q1coef, cs.q1shift, cs.q1iscale, x, gv);
        const double sq = d64[g] * r64[g];
#pragma unroll
        for (int r = 0; r < 8; ++r) x64[r * G + g] = gv[r] * sq;
      }
    }
    if (tid == 0) {
      double mn = 1e300;
      for (int c = 0; c < CS; ++c) {
        const double *rc = peer<CS>(&red[0][0], c);
        for (int w = 0; w < NW; ++w) mn = fmin(mn, rc[w]);
      }
      cs.dmin = mn;
    }
    csync<CS>();

    // interior node k -> grid index
    auto interior = [&](int k) {
      const int ix = 1 + k % m, iy = 1 + (k / m) % m, iz = 1 + k / (m * m);
      return grid3(P, ix, iy, iz);
    };

    // ---------------- right-hand sides b~ = -(A~ phi~)_I ---------------------
    {
      double bbp[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) bbp[r] = 0.0;
      for (int k = ctid; k < nI; k += CNT) {
        const int g = interior(k);
        double y[8];
        stencil27<double>(c64, x64, G, cs.offs, g, y);
        const double d = d64[g];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          r64[r * G + g] = -y[r];
          bbp[r] = fma(y[r] * d, y[r], bbp[r]);
        }
      }
      const double t = warp_transpose_reduce<8>(bbp, lane);
      if ((lane & 3) == 0) red[1][warp * 8 + (lane >> 2)] = t;
      csync<CS>();
      if (warp == 0) {
        double s = 0.0;
        for (int c = 0; c < CS; ++c) {
            const double *rc = peer<CS>(&red[1][0], c);
            for (int i = lane; i < NW * 8; i += 32) s += rc[i];
          }
#pragma unroll
        for (int mm = 8; mm < 32; mm <<= 1) s += shfl_xor_d(s, mm);
        if (lane < 8) {
          cs.bb[lane] = s;
          cs.bthr[lane] = p.tol_abs ? 1.0 : s;
        }
      }
    }
    // warm start: x~0 = D^1/2 phi_warm, r = -(A~ phi~0)_I
    if (p.warm_basis != nullptr) {
      const double *wb = p.warm_basis + (p.basis_offset ? p.basis_offset[cell] : (int64_t)cell * 8 * nn);
      csync<CS>();
      for (int k = ctid; k < nI; k += CNT) {
        const int g = interior(k);
        const int ix = 1 + k % m, iy = 1 + (k / m) % m, iz = 1 + k / (m * m);
        const int node = (iz * n + iy) * n + ix;
        const double sq = sqrt(d64[g]);
#pragma unroll
        for (int r = 0; r < 8; ++r) x64[r * G + g] = __ldg(wb + (int64_t)r * nn + node) * sq;
      }
      csync<CS>();
      for (int k = ctid; k < nI; k += CNT) {
        const int g = interior(k);
        double y[8];
        stencil27<double>(c64, x64, G, cs.offs, g, y);
#pragma unroll
        for (int r = 0; r < 8; ++r) r64[r * G + g] = -y[r];
      }
    }
    csync<CS>();
    const double tol2 = p.tol * p.tol;
    if (tid < 8) cs.inner_iters[tid] = 0;

    // 8-value block reduction finished by warp 0; returns after the barrier
    // with the totals in red[buf] lanes 0..7 read by every thread through cs
    if (!MIXED) {
      // ================= plain FP64 CG (vectors in the workspace) ==========
      // p = r on the interior, 0 on boundary and ring
      for (long i = ctid; i < 8 * G; i += CNT) p64[i] = 0.0;
      csync<CS>();
      double rp[16];
#pragma unroll
      for (int r = 0; r < 16; ++r) rp[r] = 0.0;
      for (int k = ctid; k < nI; k += CNT) {
        const int g = interior(k);
        const double d = d64[g];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          const double rv = r64[r * G + g];
          p64[r * G + g] = rv;
          rp[r] = fma(rv, rv, rp[r]);
          rp[8 + r] = fma(rv * d, rv, rp[8 + r]);
        }
      }
      {
        const double t = warp_transpose_reduce<16>(rp, lane);
        if ((lane & 1) == 0) red[0][warp * 16 + (lane >> 1)] = t;
      }
      csync<CS>();
      if (warp == 0) {
        double s = 0.0;
        for (int c = 0; c < CS; ++c) {
            const double *rc = peer<CS>(&red[0][0], c);
            for (int i = lane; i < NW * 16; i += 32) s += rc[i];
          }
        s += shfl_xor_d(s, 16);
        const double nu = shfl_xor_d(s, 8);
        if (lane < 8) {
          cs.rho[lane] = s;
          cs.active[lane] = !(nu <= tol2 * cs.bthr[lane]);
          cs.iters[lane] = 0;
        }
        __syncwarp();
        if (lane == 0) {
          int any = 0, nn2 = 0;
          for (int r = 0; r < 8; ++r) {
            any |= cs.active[r];
            if (cs.active[r] && cs.dmin * cs.rho[r] <= 100.0 * tol2 * cs.bthr[r]) nn2 = 1;
          }
          cs.done = !any;
          cs.need_nu = nn2 || p.check_interval == 1;
        }
      }
      csync<CS>();
      int it = 0;
      while (!cs.done) {
        ++it;
        double sg[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) sg[r] = 0.0;
        for (int k = ctid; k < nI; k += CNT) {
          const int g = interior(k);
          double y[8];
          stencil27<double>(c64, p64, G, cs.offs, g, y);
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            q64[r * G + g] = y[r];
            sg[r] = fma(p64[r * G + g], y[r], sg[r]);
          }
        }
        {
          const double t = warp_transpose_reduce<8>(sg, lane);
          if ((lane & 3) == 0) red[1][warp * 8 + (lane >> 2)] = t;
        }
        csync<CS>();
        if (warp == 0) {
          double s = 0.0;
          for (int c = 0; c < CS; ++c) {
            const double *rc = peer<CS>(&red[1][0], c);
            for (int i = lane; i < NW * 8; i += 32) s += rc[i];
          }
#pragma unroll
          for (int mm = 8; mm < 32; mm <<= 1) s += shfl_xor_d(s, mm);
          if (lane < 8) {
            double a = 0.0;
            if (cs.active[lane]) {
              if (cs.rho[lane] == 0.0) {
                cs.active[lane] = 0;
                cs.iters[lane] = it - 1;
              } else {
                a = cs.rho[lane] / s;
                if (!isfinite(a) || !(s > 0.0)) {
                  a = 0.0;
                  cs.active[lane] = 0;
                  cs.iters[lane] = -it;
                }
              }
            }
            cs.alpha[lane] = a;
          }
        }
        csync<CS>();
        const bool need_nu = cs.need_nu;
        double al[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) al[r] = cs.alpha[r];
#pragma unroll
        for (int r = 0; r < 16; ++r) rp[r] = 0.0;
        for (int k = ctid; k < nI; k += CNT) {
          const int g = interior(k);
          const double d = d64[g];
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            const double pv = p64[r * G + g];
            x64[r * G + g] = fma(al[r], pv, x64[r * G + g]);
            const double rv = fma(-al[r], q64[r * G + g], r64[r * G + g]);
            r64[r * G + g] = rv;
            rp[r] = fma(rv, rv, rp[r]);
            if (need_nu) rp[8 + r] = fma(rv * d, rv, rp[8 + r]);
          }
        }
        {
          const double t = warp_transpose_reduce<16>(rp, lane);
          if ((lane & 1) == 0) red[0][warp * 16 + (lane >> 1)] = t;
        }
        csync<CS>();
        if (warp == 0) {
          double s = 0.0;
          for (int c = 0; c < CS; ++c) {
            const double *rc = peer<CS>(&red[0][0], c);
            for (int i = lane; i < NW * 16; i += 32) s += rc[i];
          }
          s += shfl_xor_d(s, 16);
          const double nu = shfl_xor_d(s, 8);
          if (lane < 8) {
            double b = 0.0;
            if (cs.active[lane]) {
              if (!isfinite(s)) {
                cs.active[lane] = 0;
                cs.iters[lane] = -it;
              } else if (s == 0.0 || (need_nu && nu <= tol2 * cs.bthr[lane])) {
                cs.active[lane] = 0;
                cs.iters[lane] = it;
              } else if (it >= p.maxit) {
                cs.active[lane] = 0;
                cs.iters[lane] = -1000000 - it;
              } else {
                b = s / cs.rho[lane];
                cs.rho[lane] = s;
              }
            }
            cs.beta[lane] = b;
          }
          __syncwarp();
          if (lane == 0) {
            int any = 0, nn2 = 0;
            for (int r = 0; r < 8; ++r) {
              any |= cs.active[r];
              if (cs.active[r] && cs.dmin * cs.rho[r] <= 100.0 * tol2 * cs.bthr[r]) nn2 = 1;
            }
            cs.done = !any;
            cs.need_nu = nn2 || (p.check_interval > 0 && ((it + 1) % p.check_interval) == 0);
          }
        }
        csync<CS>();
        if (cs.done) break;
        double be[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) be[r] = cs.beta[r];
        for (int k = ctid; k < nI; k += CNT) {
          const int g = interior(k);
#pragma unroll
          for (int r = 0; r < 8; ++r) p64[r * G + g] = fma(be[r], p64[r * G + g], r64[r * G + g]);
        }
        csync<CS>();
      }
    } else {
      // ================= MIXED: FP32 inner CG + FP64 refinement ===========
      for (long i = ctid; i < 13 * G; i += CNT) c32[i] = (float)c64[i];
      for (long i = ctid; i < 8 * G; i += CNT) pp32[i] = 0.0f;
      csync<CS>();
      const float itol2 = p.inner_tol * p.inner_tol;
      int ref = 0;
      for (;;) {
        double nup[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) nup[r] = 0.0;
        for (int k = ctid; k < nI; k += CNT) {
          const int g = interior(k);
          const double d = d64[g];
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            const double rv = r64[r * G + g];
            nup[r] = fma(rv * d, rv, nup[r]);
          }
        }
        {
          const double t = warp_transpose_reduce<8>(nup, lane);
          if ((lane & 3) == 0) red[0][warp * 8 + (lane >> 2)] = t;
        }
        csync<CS>();
        if (warp == 0) {
          double s = 0.0;
          for (int c = 0; c < CS; ++c) {
            const double *rc = peer<CS>(&red[0][0], c);
            for (int i = lane; i < NW * 8; i += 32) s += rc[i];
          }
#pragma unroll
          for (int mm = 8; mm < 32; mm <<= 1) s += shfl_xor_d(s, mm);
          if (lane < 8) {
            cs.nu[lane] = s;
            if (!isfinite(s)) {
              cs.active[lane] = 0;
              cs.iters[lane] = -1;
            } else {
              cs.active[lane] = !(s <= tol2 * cs.bthr[lane]);
            }
          }
          __syncwarp();
          if (lane == 0) {
            int any = 0;
            for (int r = 0; r < 8; ++r) any |= cs.active[r];
            if (any && ref >= p.max_refine) {
              for (int r = 0; r < 8; ++r)
                if (cs.active[r]) { cs.active[r] = 0; cs.iters[r] = -1000000; }
              any = 0;
            }
            cs.done = !any;
          }
        }
        csync<CS>();
        if (cs.done) break;
        ++ref;
        float act[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) act[r] = cs.active[r] ? 1.0f : 0.0f;
        // The inner loop's FP32 vectors are node-major ([node][8 RHS], 32 B
        // per node): a thread reads a neighbour's 8 values as two 16-byte
        // loads, a warp reads 32 consecutive nodes as contiguous 1-KB runs,
        // and the 13 offsets are unrolled so their loads are in flight
        // together.
        float rho[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) rho[r] = 0.0f;
        for (int k = ctid; k < nI; k += CNT) {
          const int g = interior(k);
          float rv[8];
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            rv[r] = (float)r64[r * G + g] * act[r];
            rho[r] = fmaf(rv[r], rv[r], rho[r]);
          }
          st8(rr32, g, rv);
          st8(pp32, g, rv);
          const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
          st8(dd32, g, z);
        }
        int buf = 0;
        auto block_sum8 = [&](float (&v)[8]) {
          float vv[8];
#pragma unroll
          for (int r = 0; r < 8; ++r) vv[r] = v[r];
          const float t = warp_transpose_reduce<8>(vv, lane);
          float *rb = reinterpret_cast<float *>(red[buf]);
          if ((lane & 3) == 0) rb[warp * 8 + (lane >> 2)] = t;
          csync<CS>();
          float s = 0.f;
          for (int c = 0; c < CS; ++c) {
            const float *rc = peer<CS>(rb, c);
            for (int i = lane; i < NW * 8; i += 32) s += rc[i];
          }
#pragma unroll
          for (int mm = 8; mm < 32; mm <<= 1) s += shfl_xor_d(s, mm);
#pragma unroll
          for (int r = 0; r < 8; ++r) v[r] = __shfl_sync(0xffffffffu, s, r);
          buf ^= 1;
        };
        block_sum8(rho);
        // stopping threshold on r.r per RHS and the active set as a bit mask
        // (few registers: the 2-CTA/SM shapes run at 64 per thread)
        float thr[8];
        unsigned iact = 0u;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          if (act[r] > 0.0f && rho[r] > 0.0f) iact |= 1u << r;
          // never deeper than the outer goal needs (factor 10 margin)
          const double goal = cs.nu[r] > 0.0 ? 0.01 * tol2 * cs.bthr[r] / cs.nu[r] : 0.0;
          thr[r] = fmaxf(itol2, (float)fmin(goal, 0.25)) * rho[r];
        }
        if (tid < 8) {
          float t = 0.f, q = 0.f;
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            t = r == tid ? thr[r] : t;
            q = r == tid ? rho[r] : q;
          }
          cs.seg_thr[tid] = t;
          cs.seg_rho[0][tid] = q;
        }
        __syncthreads();
        // N = 8, 16, 24 (the uneven 3D sphere workload) get the z-pair stencil
        // with compile-time offsets
        if constexpr (CS > 1) {
          // cluster shape: the slabs of the cell stay in the CTAs' shared memory
          inner_segment3d_slab<NT, CS, (kNMax3D - 1 + CS - 1) / CS>(c32, rr32, dd32, G, N, P, p.inner_maxit, iact,
                                                                   reinterpret_cast<float *>(red[0]), cs, dsm3);
        } else if (N == 24) {
          inner_segment3d<NT, CS, 27>(c32, pp32, qq32, rr32, dd32, G, m, P, nI, p.inner_maxit, iact, buf, red, cs);
        } else if (N == 16) {
          inner_segment3d<NT, CS, 19>(c32, pp32, qq32, rr32, dd32, G, m, P, nI, p.inner_maxit, iact, buf, red, cs);
        } else if (N == 8) {
          inner_segment3d<NT, CS, 11>(c32, pp32, qq32, rr32, dd32, G, m, P, nI, p.inner_maxit, iact, buf, red, cs);
        } else {
          inner_segment3d<NT, CS, 0>(c32, pp32, qq32, rr32, dd32, G, m, P, nI, p.inner_maxit, iact, buf, red, cs);
        }
        // x~ += d (FP64); r = -(A~ phi~)_I in FP64
        for (int k = ctid; k < nI; k += CNT) {
          const int g = interior(k);
          float dv[8];
          ld8(dd32, g, dv);
#pragma unroll
          for (int r = 0; r < 8; ++r) x64[r * G + g] += (double)dv[r];
        }
        csync<CS>();
        for (int k = ctid; k < nI; k += CNT) {
          const int g = interior(k);
          double y[8];
          stencil27<double>(c64, x64, G, cs.offs, g, y);
#pragma unroll
          for (int r = 0; r < 8; ++r) r64[r * G + g] = -y[r];
        }
        csync<CS>();
      }
      if (tid == 0) cs.refinements = ref;
      csync<CS>();
    }

    agree_status();
    // ---------------- epilogue: M (64), F (8), true residual (8) -----------
    // x64 holds phi~ (the boundary values were never overwritten)
    const double fj = p.f_value;
    for (int part = 0; part < 3; ++part) {
      double acc[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) acc[i] = 0.0;
      for (int k = ctid; k < nn; k += CNT) {
        const int ix = k % n, iy = (k / n) % n, iz = k / (n * n);
        const int g = grid3(P, ix, iy, iz);
        if (part < 2) {
          double y[8];
          const bool inner = ix > 0 && iy > 0 && iz > 0 && ix < N && iy < N && iz < N;
          if (MIXED && inner) {
            // interior rows: A~ phi~ = -r, the FP64 residual of the final
            // iterate (computed after the last correction)
#pragma unroll
            for (int r = 0; r < 8; ++r) y[r] = -r64[r * G + g];
          } else {
            stencil27<double>(c64, x64, G, cs.offs, g, y);
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const double ph = x64[(long)(4 * part + i) * G + g];
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[8 * i + j] = fma(ph, y[j], acc[8 * i + j]);
          }
        } else {
          // load vector b_k (affine: f |det| / 8 per adjacent fine cell)
          // b_k = int f psi_k (diffusion_problem_basis.tpp:219-220)
          double bl;
          if (cs.affine && !p.f_qp) {
            const double mult = (ix == 0 || ix == N ? 1.0 : 2.0) * (iy == 0 || iy == N ? 1.0 : 2.0) *
                                (iz == 0 || iz == N ? 1.0 : 2.0);
            bl = fj * 0.125 * cs.absdet * mult;
          } else {
            // QGauss(2) over the adjacent fine cells: f tabulated at the Gauss
            // points (p.f_qp) or constant; per-point |det J| on general cells
            const double invN = 1.0 / (double)N;
            const int nfc = N * N * N;
            const double *fq =
                p.f_qp ? p.f_qp + (p.f_qp_offset ? p.f_qp_offset[cell] : (int64_t)cell * 8 * nfc) : nullptr;
            bl = 0.0;
            for (int c8 = 0; c8 < 8; ++c8) {
              const int cx = ix - (c8 & 1), cy = iy - ((c8 >> 1) & 1), cz = iz - (c8 >> 2);
              if (cx < 0 || cy < 0 || cz < 0 || cx >= N || cy >= N || cz >= N) continue;
              const int kv = (c8 & 1) + 2 * ((c8 >> 1) & 1) + 4 * (c8 >> 2);  // local vertex
              const int fc = (cz * N + cy) * N + cx;
              double V[24];
              if (!cs.affine)
                for (int k8 = 0; k8 < 8; ++k8) {
                  const double t[3] = {(cx + (k8 & 1)) * invN, (cy + ((k8 >> 1) & 1)) * invN, (cz + (k8 >> 2)) * invN};
                  trilinear_map(cs.corners, t, V + 3 * k8);
                }
              for (int q = 0; q < 8; ++q) {
                double det = cs.absdet;
                if (!cs.affine) {
                  double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                  for (int k8 = 0; k8 < 8; ++k8)
                    for (int a = 0; a < 3; ++a)
                      for (int c = 0; c < 3; ++c) J[3 * a + c] += V[3 * k8 + a] * rgrad(k8, q, c);
                  det = fabs(J[0] * (J[4] * J[8] - J[5] * J[7]) + J[1] * (J[5] * J[6] - J[3] * J[8]) +
                             J[2] * (J[3] * J[7] - J[4] * J[6]));
                }
                const double psi = lv3(kv & 1, q & 1) * lv3((kv >> 1) & 1, (q >> 1) & 1) * lv3(kv >> 2, q >> 2);
                const double f = fq ? fq[q * nfc + fc] : fj;
                bl += f * psi * 0.125 * det;
              }
            }
          }
          const double d = d64[g];
          const double s = rsqrt(d);
#pragma unroll
          for (int i = 0; i < 8; ++i) acc[i] = fma(x64[(long)i * G + g], bl * s, acc[i]);
          // true residual norm (the mixed form has it from its last check)
          if (!MIXED && ix > 0 && iy > 0 && iz > 0 && ix < N && iy < N && iz < N) {
            double y[8];
            stencil27<double>(c64, x64, G, cs.offs, g, y);
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[8 + j] = fma(y[j] * d, y[j], acc[8 + j]);
          }
          if (p.basis) {
            double *out = p.basis + (p.basis_offset ? p.basis_offset[cell] : (int64_t)cell * 8 * nn);
#pragma unroll
            for (int i = 0; i < 8; ++i) out[(int64_t)i * nn + k] = x64[(long)i * G + g] * s;
          }
        }
      }
      const double tot = warp_transpose_reduce<32>(acc, lane);
      redE[warp * 32 + lane] = tot;
      csync<CS>();
      if (warp == 0 && crank == 0) {
        double s = 0.0;
        for (int c = 0; c < CS; ++c) {
          const double *rc = peer<CS>(&redE[0], c);
          for (int w = 0; w < NW; ++w) s += rc[w * 32 + lane];
        }
        if (part < 2) {
          p.M[(int64_t)cell * 64 + part * 32 + lane] = s;
        } else {
          if (lane < 8) p.F[(int64_t)cell * 8 + lane] = s;
          double rel = 0.0;
          if (lane >= 8 && lane < 16) {
            const double bb = cs.bb[lane - 8];
            const double nu = MIXED ? cs.nu[lane - 8] : s;
            rel = bb > 0.0 ? sqrt(nu / bb) : sqrt(nu);
          }
#pragma unroll
          for (int mm = 16; mm >= 1; mm >>= 1) rel = fmax(rel, shfl_xor_d(rel, mm));
          if (lane < 8 && p.iters) {
            const int itv = cs.iters[lane];
            p.iters[(int64_t)cell * 8 + lane] =
                MIXED ? cs.inner_iters[lane] : (itv >= 0 ? itv : (itv <= -1000000 ? -itv - 1000000 : -itv));
          }
          if (lane == 0) {
            int st = cs.status;
            for (int r = 0; r < 8; ++r) {
              const int itv = cs.iters[r];
              if (itv <= -1000000) st = st == MSFEM_CELL_CONVERGED ? MSFEM_CELL_MAXIT : st;
              else if (itv < 0) st = MSFEM_CELL_NAN;
            }
            if (!isfinite(rel)) st = MSFEM_CELL_NAN;
            p.status[cell] = st;
            if (p.rel_res) p.rel_res[cell] = rel;
            if (p.refinements) p.refinements[cell] = cs.refinements;
          }
        }
      }
      csync<CS>();
    }
  }
}

// Energy norms against a reference basis (3D): err[cell][i] = ||phi_i - ref_i||_A,
// nrm[cell][i] = ||ref_i||_A, element by element over the fine hexahedra;
// bases in the basis-output layout ([cell][8][(N+1)^3], lexicographic nodes).
template <int NT>
__global__ void __launch_bounds__(NT)
msfem3d_energy_kernel(const KernelParams p, const double *__restrict__ basis,
                      const double *__restrict__ ref, double *__restrict__ err,
                      double *__restrict__ nrm) {
  constexpr int NW = NT / 32;
  __shared__ CellShared3D cs;
  __shared__ double red[NW * 16];
  __shared__ int bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool scalar = (p.coef_kind == MSFEM_COEF_TABULATED && p.ncomp == 1) ||
                      p.coef_kind == MSFEM_COEF_SINSIN;
  for (int cell = blockIdx.x; cell < p.n_cells; cell += gridDim.x) {
    const int N = p.n_fine ? p.n_fine[cell] : p.n_fine_uniform;
    if (tid == 0) bad = 0;
    cell_geometry3d<NT>(p, cs, cell, N, scalar, tid);
    const int st = cs.status;
    double acc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = 0.0;
    if (st == MSFEM_CELL_CONVERGED) {
      const int n = N + 1, nn = n * n * n, nfc = N * N * N;
      const int64_t off = p.basis_offset ? p.basis_offset[cell] : (int64_t)cell * 8 * nn;
      const double *a = basis + off, *r = ref + off;
      const double *tab = nullptr;
      if (p.coef_kind == MSFEM_COEF_TABULATED)
        tab = p.qp_values + (p.qp_offset ? p.qp_offset[cell] : (int64_t)cell * p.ncomp * 8 * nfc);
      const bool need_x = p.coef_kind != MSFEM_COEF_TABULATED && p.coef_kind != MSFEM_COEF_CONSTANT;
      for (int fc = tid; fc < nfc; fc += NT) {
        const int cx = fc % N, cy = (fc / N) % N, cz = fc / (N * N);
        double K[36];
        if (!element3d(p, cs, tab, N, cx, cy, cz, scalar, need_x, K)) bad = 1;
        int kk[8];
#pragma unroll
        for (int v = 0; v < 8; ++v)
          kk[v] = (cx + (v & 1)) + n * ((cy + ((v >> 1) & 1)) + n * (cz + (v >> 2)));
#pragma unroll 1
        for (int i = 0; i < 8; ++i) {
          double e[8], w[8];
#pragma unroll
          for (int v = 0; v < 8; ++v) {
            w[v] = r[(int64_t)i * nn + kk[v]];
            e[v] = a[(int64_t)i * nn + kk[v]] - w[v];
          }
          double qe = 0.0, qw = 0.0;
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            double se = 0.5 * K[tri_index(u, u)] * e[u], sw = 0.5 * K[tri_index(u, u)] * w[u];
#pragma unroll
            for (int v = u + 1; v < 8; ++v) {
              se = fma(K[tri_index(u, v)], e[v], se);
              sw = fma(K[tri_index(u, v)], w[v], sw);
            }
            qe = fma(e[u], se, qe);
            qw = fma(w[u], sw, qw);
          }
          // acc[i] is the register array index; i is not unrolled, so select
#pragma unroll
          for (int j = 0; j < 8; ++j)
            if (j == i) { acc[j] += 2.0 * qe; acc[8 + j] += 2.0 * qw; }
        }
      }
    }
    warp_partials<16>(acc, red, warp, lane);
    __syncthreads();
    if (warp == 0) {
      const double s = warp_finish<16>(red, NW, lane);
      if (lane < 16) {
        double out = sqrt(fmax(s, 0.0));
        if (st != MSFEM_CELL_CONVERGED || bad || !isfinite(s)) out = __longlong_as_double(0x7ff8000000000000ll);
        (lane < 8 ? err : nrm)[(int64_t)cell * 8 + (lane & 7)] = out;
      }
    }
    __syncthreads();
  }
}

}  // namespace msfem
