// msfem_kernel2d.cuh -- 2D multiscale-basis kernel for sm_103a.
//
// One CTA owns one coarse cell at a time (persistent CTAs pull cells from a
// work queue).  Per cell, entirely in shared memory:
//   1. assemble the fine Q1 stiffness (QGauss(2)) as a 9-point node stencil,
//      4-colour scatter, no atomics (diffusion_problem_basis.tpp:159-242);
//   2. scale it symmetrically by D^-1/2 (unit diagonal): Jacobi-preconditioned
//      CG becomes plain CG on  A~ = D^-1/2 A D^-1/2;
//   3. solve the 4 Dirichlet problems A_II u_i = -A_IB g_i together, g_i the
//      coarse Q1 nodal functions (diffusion_problem_basis.tpp:450-465,
//      basis_q1.tpp), with a per-RHS relative l2 stopping rule;
//   4. epilogue M_ij = phi_i^T A phi_j and F_i = phi_i^T b over all fine nodes
//      (diffusion_problem_basis.tpp:245-285) -- in scaled form
//      M_ij = phi~_i^T A~ phi~_j with phi~ = D^1/2 phi.
//
// Precision forms:
//   FP64  : plain FP64 CG (the drop-in form).
//   MIXED : FP64 outer loop  r = b - A x  (true FP64 residual), inner FP32 CG
//           on A~ d = r to a relative reduction, x += d in FP64.
//
// Shared-memory layout (node-major, 4 values per node; P = N + 3: the
// (N+1)^2 node grid plus a zero ring, node (ix,iy) at (iy+1) P + ix + 1):
//   c64 [G][4]  scaled couplings E, NE, N, NW of each node (FP64)
//   v64 [G][4]  FP64 work vector of the 4 RHS (p~ in FP64 CG, phi~ otherwise)
//   s64 [G]     D^-1/2,  d64 [G] D (diagonal),  bl64 [G] D^-1/2 b_load
//   c32 [G][4], v32 [G][4]   FP32 copies for the MIXED inner loop
#pragma once

#include "msfem_common.cuh"

namespace msfem {

template <int NMAX>
struct Smem2D {
  static constexpr int P = NMAX + 3;
  static constexpr int G = P * P;
  // every array starts on a 128-byte boundary (vector loads need 16 B)
  static constexpr size_t al(size_t x) { return (x + 127) & ~size_t(127); }
  static constexpr size_t kC64 = 0;
  static constexpr size_t kV64 = al(kC64 + sizeof(double) * 4 * G);
  static constexpr size_t kS64 = al(kV64 + sizeof(double) * 4 * G);
  static constexpr size_t kD64 = al(kS64 + sizeof(double) * G);
  static constexpr size_t kB64 = al(kD64 + sizeof(double) * G);
  static constexpr size_t kEndFP64 = al(kB64 + sizeof(double) * G);
  static constexpr size_t kC32 = kEndFP64;
  static constexpr size_t kV32 = al(kC32 + sizeof(float) * 4 * G);
  static constexpr size_t kEndMixed = al(kV32 + sizeof(float) * 4 * G);
  static constexpr size_t bytes(bool mixed) { return mixed ? kEndMixed : kEndFP64; }
  static_assert(kV64 % 16 == 0 && kC32 % 16 == 0 && kV32 % 16 == 0, "vector alignment");
};

__device__ __forceinline__ void ld4(const double *__restrict__ v, int g, double (&t)[4]) {
  const double2 a = *reinterpret_cast<const double2 *>(v + 4 * g);
  const double2 b = *reinterpret_cast<const double2 *>(v + 4 * g + 2);
  t[0] = a.x; t[1] = a.y; t[2] = b.x; t[3] = b.y;
}
__device__ __forceinline__ void st4(double *__restrict__ v, int g, const double (&t)[4]) {
  *reinterpret_cast<double2 *>(v + 4 * g) = make_double2(t[0], t[1]);
  *reinterpret_cast<double2 *>(v + 4 * g + 2) = make_double2(t[2], t[3]);
}
__device__ __forceinline__ void ld4(const float *__restrict__ v, int g, float (&t)[4]) {
  const float4 a = *reinterpret_cast<const float4 *>(v + 4 * g);
  t[0] = a.x; t[1] = a.y; t[2] = a.z; t[3] = a.w;
}
__device__ __forceinline__ void st4(float *__restrict__ v, int g, const float (&t)[4]) {
  *reinterpret_cast<float4 *>(v + 4 * g) = make_float4(t[0], t[1], t[2], t[3]);
}

// y = A~ v at node g (unit diagonal + 8 scaled couplings), 4 RHS.
template <typename T>
__device__ __forceinline__ void stencil9(const T *__restrict__ c, const T *__restrict__ v,
                                         int g, int P, T (&y)[4]) {
  T cc[4], t[4];
  ld4(c, g, cc);
  const T cW = c[4 * (g - 1) + 0];
  const T cS = c[4 * (g - P) + 2];
  const T cSW = c[4 * (g - P - 1) + 1];
  const T cSE = c[4 * (g - P + 1) + 3];
  ld4(v, g, y);
#define MSFEM_ACC(OFF, COEF)                      \
  ld4(v, g + (OFF), t);                           \
  _Pragma("unroll") for (int r = 0; r < 4; ++r) y[r] = fma(COEF, t[r], y[r]);
  MSFEM_ACC(1, cc[0])
  MSFEM_ACC(-1, cW)
  MSFEM_ACC(P, cc[2])
  MSFEM_ACC(-P, cS)
  MSFEM_ACC(P + 1, cc[1])
  MSFEM_ACC(-P - 1, cSW)
  MSFEM_ACC(P - 1, cc[3])
  MSFEM_ACC(-P + 1, cSE)
#undef MSFEM_ACC
}

// Warp 0 finishes a K-value block reduction: red holds NW*K warp partials
// ([warp][value]); on return lane l holds the block total of value l % K.
template <int K, typename T>
__device__ __forceinline__ T warp0_finish(const T *red, int NW, int lane) {
  T s = T(0);
  for (int i = lane; i < NW * K; i += 32) s += red[i];
#pragma unroll
  for (int m = K; m < 32; m <<= 1) s += shfl_xor_d(s, m);
  return s;
}

// Per-warp partials of a K-value reduction into red[warp][K].
template <int K, typename T>
__device__ __forceinline__ void warp_partials(T (&vals)[K], T *red, int warp, int lane) {
  const T tot = warp_transpose_reduce<K>(vals, lane);
  constexpr int SPAN = 32 / K;
  if ((lane & (SPAN - 1)) == 0) red[warp * K + lane / SPAN] = tot;
}

// Block-uniform scalars of one cell, in shared memory.
struct CellShared2D {
  double corners[8];
  double q1coef[16];
  double q1shift[2];
  double q1iscale;
  double jinv_g[9];   // affine cells: G = w|det| Jinv A Jinv^T as 3x3 map (a11,a12,a22) -> (G11,G12,G22)
  double jfine[4];    // affine cells: fine-cell Jacobian (column-major dx/dxi, dx/deta)
  double absdet;      // affine cells: |det J_fine|
  double bb[4];       // ||b_i||^2 (unscaled)
  double rho[4];
  double alpha[4];
  double beta[4];
  double dmin;
  float alpha32[4];
  int active[4];
  int iters[4];
  int status;
  int affine;
  int need_nu;
  int done;
  int cell;
  int refinements;
};

__device__ __forceinline__ void bilinear_map(const double *cr, double tx, double ty, double *x) {
  const double w0 = (1.0 - tx) * (1.0 - ty), w1 = tx * (1.0 - ty);
  const double w2 = (1.0 - tx) * ty, w3 = tx * ty;
  x[0] = w0 * cr[0] + w1 * cr[2] + w2 * cr[4] + w3 * cr[6];
  x[1] = w0 * cr[1] + w1 * cr[3] + w2 * cr[5] + w3 * cr[7];
}

// QGauss(2) on [0,1]: (1 -+ 1/sqrt(3))/2
__device__ __forceinline__ double gauss2(int i) {
  return i ? 0.78867513459481288225457439025098 : 0.21132486540518711774542560974902;
}
// l_b(gauss2(qb)),  l_0(t) = 1 - t,  l_1(t) = t
__device__ __forceinline__ double lval(int b, int qb) {
  return b ? gauss2(qb) : gauss2(1 - qb);
}

template <int NMAX, int NT, bool MIXED>
__global__ void __launch_bounds__(NT, MIXED ? 1 : 2)
msfem2d_kernel(const KernelParams p) {
  using L = Smem2D<NMAX>;
  constexpr int NW = NT / 32;
  constexpr int NPT = ((NMAX - 1) * (NMAX - 1) + NT - 1) / NT;  // interior nodes per thread
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *c64 = reinterpret_cast<double *>(smem_raw + L::kC64);
  double *v64 = reinterpret_cast<double *>(smem_raw + L::kV64);
  double *s64 = reinterpret_cast<double *>(smem_raw + L::kS64);
  double *d64 = reinterpret_cast<double *>(smem_raw + L::kD64);
  double *b64 = reinterpret_cast<double *>(smem_raw + L::kB64);
  float *c32 = reinterpret_cast<float *>(smem_raw + L::kC32);
  float *v32 = reinterpret_cast<float *>(smem_raw + L::kV32);
  __shared__ CellShared2D cs;
  __shared__ double red[2][NW * 32];
  __shared__ float red32[2][NW * 8];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (;;) {
    if (tid == 0) {
      const unsigned wi = atomicAdd(p.queue, 1u);
      cs.cell = wi < (unsigned)p.n_cells ? (p.order ? p.order[wi] : (int)wi) : -1;
    }
    __syncthreads();
    const int cell = cs.cell;
    if (cell < 0) break;
    const int N = p.n_fine ? p.n_fine[cell] : p.n_fine_uniform;
    const int P = N + 3, G = P * P, n = N + 1, nI = (N - 1) * (N - 1);

    // ---------------- set-up -------------------------------------------
    if (tid < 8) cs.corners[tid] = p.corners[(int64_t)cell * 8 + tid];
    for (int i = tid; i < 4 * G; i += NT) { c64[i] = 0.0; v64[i] = 0.0; }
    for (int i = tid; i < G; i += NT) { s64[i] = 0.0; d64[i] = 0.0; b64[i] = 0.0; }
    if (MIXED)
      for (int i = tid; i < 4 * G; i += NT) { c32[i] = 0.0f; v32[i] = 0.0f; }
    if (tid < 4) { cs.iters[tid] = 0; cs.active[tid] = 1; }
    __syncthreads();
    if (tid == 0) {
      const double *cr = cs.corners;
      int st = MSFEM_CELL_CONVERGED;
      if (N < 1 || N > NMAX) st = MSFEM_CELL_BAD_INPUT;
      if (!q1_setup<2>(cr, cs.q1coef, cs.q1shift, &cs.q1iscale)) st = MSFEM_CELL_BAD_INPUT;
      // parallelogram test v0 + v3 == v1 + v2 (exact)
      const int aff = (cr[0] + cr[6] == cr[2] + cr[4]) && (cr[1] + cr[7] == cr[3] + cr[5]);
      cs.affine = aff;
      if (aff && st == MSFEM_CELL_CONVERGED) {
        const double invN = 1.0 / (double)N;
        const double J00 = (cr[2] - cr[0]) * invN, J10 = (cr[3] - cr[1]) * invN;
        const double J01 = (cr[4] - cr[0]) * invN, J11 = (cr[5] - cr[1]) * invN;
        const double det = J00 * J11 - J01 * J10;
        if (!(det > 0.0)) st = MSFEM_CELL_BAD_INPUT;
        const double id = 1.0 / det;
        const double i00 = J11 * id, i01 = -J01 * id, i10 = -J10 * id, i11 = J00 * id;
        const double w = 0.25 * fabs(det);
        // G = w Ji A Ji^T,  A = [[a11,a12],[a12,a22]]
        cs.jinv_g[0] = w * i00 * i00; cs.jinv_g[1] = w * 2.0 * i00 * i01; cs.jinv_g[2] = w * i01 * i01;
        cs.jinv_g[3] = w * i00 * i10; cs.jinv_g[4] = w * (i00 * i11 + i01 * i10); cs.jinv_g[5] = w * i01 * i11;
        cs.jinv_g[6] = w * i10 * i10; cs.jinv_g[7] = w * 2.0 * i10 * i11; cs.jinv_g[8] = w * i11 * i11;
        cs.jfine[0] = J00; cs.jfine[1] = J10; cs.jfine[2] = J01; cs.jfine[3] = J11;
        cs.absdet = fabs(det);
      }
      cs.status = st;
    }
    __syncthreads();
    if (cs.status != MSFEM_CELL_CONVERGED) {
      // malformed cell: report and move on (outputs NaN)
      if (tid < 16) p.M[(int64_t)cell * 16 + tid] = __longlong_as_double(0x7ff8000000000000ll);
      if (tid < 4) {
        p.F[(int64_t)cell * 4 + tid] = __longlong_as_double(0x7ff8000000000000ll);
        if (p.iters) p.iters[(int64_t)cell * 4 + tid] = 0;
      }
      if (tid == 0) {
        p.status[cell] = cs.status;
        if (p.rel_res) p.rel_res[cell] = __longlong_as_double(0x7ff8000000000000ll);
        if (p.refinements) p.refinements[cell] = 0;
      }
      __syncthreads();
      continue;
    }

    // ---------------- assembly: 4-colour scatter -------------------------
    {
      const int nfc = N * N;
      const double *tab = nullptr;
      if (p.coef_kind == MSFEM_COEF_TABULATED)
        tab = p.qp_values + (p.qp_offset ? p.qp_offset[cell] : (int64_t)cell * p.ncomp * 4 * nfc);
      const double invN = 1.0 / (double)N;
      const bool need_x = p.coef_kind != MSFEM_COEF_TABULATED && p.coef_kind != MSFEM_COEF_CONSTANT;
      for (int col = 0; col < 4; ++col) {
        const int ox = col & 1, oy = col >> 1;
        const int nx = (N - ox + 1) >> 1, ny = (N - oy + 1) >> 1;
        for (int idx = tid; idx < nx * ny; idx += NT) {
          const int cx = ox + 2 * (idx % nx), cy = oy + 2 * (idx / nx);
          const int fc = cx + N * cy;
          double K[4][4];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) K[i][j] = 0.0;
          double bload[4] = {0.0, 0.0, 0.0, 0.0};
          bool bad = false;
          double V[8];
          if (!cs.affine) {
            bilinear_map(cs.corners, cx * invN, cy * invN, V + 0);
            bilinear_map(cs.corners, (cx + 1) * invN, cy * invN, V + 2);
            bilinear_map(cs.corners, cx * invN, (cy + 1) * invN, V + 4);
            bilinear_map(cs.corners, (cx + 1) * invN, (cy + 1) * invN, V + 6);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int qx = q & 1, qy = q >> 1;
            const double xi = gauss2(qx), eta = gauss2(qy);
            double xq[2] = {0.0, 0.0};
            double Gm[3];
            double A[3];
            if (cs.affine) {
              if (need_x) {
                const double u = cx + xi, v = cy + eta;
                xq[0] = cs.corners[0] + cs.jfine[0] * u + cs.jfine[2] * v;
                xq[1] = cs.corners[1] + cs.jfine[1] * u + cs.jfine[3] * v;
              }
              coef_at<2>(p, xq, tab, q, nfc, fc, A);
              Gm[0] = cs.jinv_g[0] * A[0] + cs.jinv_g[1] * A[1] + cs.jinv_g[2] * A[2];
              Gm[1] = cs.jinv_g[3] * A[0] + cs.jinv_g[4] * A[1] + cs.jinv_g[5] * A[2];
              Gm[2] = cs.jinv_g[6] * A[0] + cs.jinv_g[7] * A[1] + cs.jinv_g[8] * A[2];
              const double wf = 0.25 * cs.absdet * p.f_value;
#pragma unroll
              for (int k = 0; k < 4; ++k) bload[k] += wf * lval(k & 1, qx) * lval(k >> 1, qy);
            } else {
              // J = sum_k V_k (x) grad psi_k(xi, eta)
              double J00 = 0, J01 = 0, J10 = 0, J11 = 0;
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                const int kx = k & 1, ky = k >> 1;
                const double gx = (kx ? 1.0 : -1.0) * lval(ky, qy);
                const double gy = (ky ? 1.0 : -1.0) * lval(kx, qx);
                const double psi = lval(kx, qx) * lval(ky, qy);
                J00 += V[2 * k] * gx; J01 += V[2 * k] * gy;
                J10 += V[2 * k + 1] * gx; J11 += V[2 * k + 1] * gy;
                xq[0] += psi * V[2 * k]; xq[1] += psi * V[2 * k + 1];
              }
              const double det = J00 * J11 - J01 * J10;
              if (!(det > 0.0)) bad = true;
              const double id = 1.0 / det;
              const double i00 = J11 * id, i01 = -J01 * id, i10 = -J10 * id, i11 = J00 * id;
              const double w = 0.25 * fabs(det);
              coef_at<2>(p, xq, tab, q, nfc, fc, A);
              // T = Ji A, G = T Ji^T
              const double t00 = i00 * A[0] + i01 * A[1], t01 = i00 * A[1] + i01 * A[2];
              const double t10 = i10 * A[0] + i11 * A[1], t11 = i10 * A[1] + i11 * A[2];
              Gm[0] = w * (t00 * i00 + t01 * i01);
              Gm[1] = w * (t00 * i10 + t01 * i11);
              Gm[2] = w * (t10 * i10 + t11 * i11);
#pragma unroll
              for (int k = 0; k < 4; ++k)
                bload[k] += w * p.f_value * lval(k & 1, qx) * lval(k >> 1, qy);
            }
            // reference gradients at this Gauss point
            double gx[4], gy[4], ax[4], ay[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int kx = k & 1, ky = k >> 1;
              gx[k] = (kx ? 1.0 : -1.0) * lval(ky, qy);
              gy[k] = (ky ? 1.0 : -1.0) * lval(kx, qx);
              ax[k] = Gm[0] * gx[k] + Gm[1] * gy[k];
              ay[k] = Gm[1] * gx[k] + Gm[2] * gy[k];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = i; j < 4; ++j) K[i][j] = fma(gx[i], ax[j], fma(gy[i], ay[j], K[i][j]));
          }
          if (bad) cs.status = MSFEM_CELL_BAD_INPUT;
          const int g0 = (cy + 1) * P + cx + 1;
          const int g1 = g0 + 1, g2 = g0 + P, g3 = g0 + P + 1;
          d64[g0] += K[0][0]; d64[g1] += K[1][1]; d64[g2] += K[2][2]; d64[g3] += K[3][3];
          c64[4 * g0 + 0] += K[0][1];  // E  of node 0
          c64[4 * g2 + 0] += K[2][3];  // E  of node 2
          c64[4 * g0 + 2] += K[0][2];  // N  of node 0
          c64[4 * g1 + 2] += K[1][3];  // N  of node 1
          c64[4 * g0 + 1] += K[0][3];  // NE of node 0
          c64[4 * g1 + 3] += K[1][2];  // NW of node 1
          b64[g0] += bload[0]; b64[g1] += bload[1]; b64[g2] += bload[2]; b64[g3] += bload[3];
        }
        __syncthreads();
      }
    }
    if (cs.status != MSFEM_CELL_CONVERGED) {
      if (tid < 16) p.M[(int64_t)cell * 16 + tid] = __longlong_as_double(0x7ff8000000000000ll);
      if (tid < 4) {
        p.F[(int64_t)cell * 4 + tid] = __longlong_as_double(0x7ff8000000000000ll);
        if (p.iters) p.iters[(int64_t)cell * 4 + tid] = 0;
      }
      if (tid == 0) {
        p.status[cell] = cs.status;
        if (p.rel_res) p.rel_res[cell] = __longlong_as_double(0x7ff8000000000000ll);
        if (p.refinements) p.refinements[cell] = 0;
      }
      __syncthreads();
      continue;
    }

    // ---------------- symmetric scaling ----------------------------------
    for (int k = tid; k < n * n; k += NT) {
      const int g = (k / n + 1) * P + k % n + 1;
      const double d = d64[g];
      const double s = rsqrt(d);
      s64[g] = s;
      b64[g] *= s;
    }
    __syncthreads();
    double dmin_part = 1e300;
    for (int k = tid; k < n * n; k += NT) {
      const int ix = k % n, iy = k / n;
      const int g = (iy + 1) * P + ix + 1;
      const double s = s64[g];
      double cc[4];
      ld4(c64, g, cc);
      cc[0] *= s * s64[g + 1];
      cc[1] *= s * s64[g + P + 1];
      cc[2] *= s * s64[g + P];
      cc[3] *= s * s64[g + P - 1];
      st4(c64, g, cc);
      if (MIXED) {
        float cf[4] = {(float)cc[0], (float)cc[1], (float)cc[2], (float)cc[3]};
        st4(c32, g, cf);
      }
      const bool bnd = ix == 0 || iy == 0 || ix == N || iy == N;
      const double d = d64[g];
      if (bnd) {
        // Dirichlet data phi~_i = D^1/2 g_i (BasisQ1 at the node)
        double x[2], gv[4];
        bilinear_map(cs.corners, ix / (double)N, iy / (double)N, x);
        q1_eval<2>(cs.q1coef, cs.q1shift, cs.q1iscale, x, gv);
        const double sq = d * s;
        double t[4] = {gv[0] * sq, gv[1] * sq, gv[2] * sq, gv[3] * sq};
        st4(v64, g, t);
      } else {
        dmin_part = fmin(dmin_part, d);
        if (!(d > 0.0) || !isfinite(d)) cs.status = MSFEM_CELL_NAN;
      }
    }
    // dmin (block min)
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) dmin_part = fmin(dmin_part, shfl_xor_d(dmin_part, m));
    if (lane == 0) red[0][warp] = dmin_part;
    __syncthreads();
    if (tid == 0) {
      double m = 1e300;
      for (int w = 0; w < NW; ++w) m = fmin(m, red[0][w]);
      cs.dmin = m;
    }

    // ---------------- right-hand sides ------------------------------------
    int gidx[NPT];
    double dloc[NPT];
#pragma unroll
    for (int j = 0; j < NPT; ++j) {
      const int k = tid + j * NT;
      gidx[j] = k < nI ? (1 + k / (N - 1) + 1) * P + (1 + k % (N - 1)) + 1 : -1;
      dloc[j] = gidx[j] >= 0 ? d64[gidx[j]] : 0.0;
    }
    double rr[NPT][4];   // FP64 residual (scaled)
    double bbp[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int j = 0; j < NPT; ++j) {
#pragma unroll
      for (int r = 0; r < 4; ++r) rr[j][r] = 0.0;
      if (gidx[j] >= 0) {
        double y[4];
        stencil9<double>(c64, v64, gidx[j], P, y);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          rr[j][r] = -y[r];
          bbp[r] = fma(rr[j][r] * dloc[j], rr[j][r], bbp[r]);
        }
      }
    }
    warp_partials<4>(bbp, red[1], warp, lane);
    __syncthreads();
    if (warp == 0) {
      const double t = warp0_finish<4>(red[1], NW, lane);
      if (lane < 4) cs.bb[lane] = t;
    }
    // warm start: x~0 = D^1/2 phi_warm on the interior, r0 = -(A~ phi~0)_I
    const bool warm = p.warm_basis != nullptr;
    if (warm) {
      const double *wb = p.warm_basis + (p.basis_offset ? p.basis_offset[cell] : (int64_t)cell * 4 * n * n);
      __syncthreads();
#pragma unroll
      for (int j = 0; j < NPT; ++j)
        if (gidx[j] >= 0) {
          const int g = gidx[j];
          const int node = (g / P - 1) * n + (g % P - 1);
          const double sq = d64[g] * s64[g];
          double t[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) t[r] = __ldg(wb + (int64_t)r * n * n + node) * sq;
          st4(v64, g, t);
        }
      __syncthreads();
#pragma unroll
      for (int j = 0; j < NPT; ++j)
        if (gidx[j] >= 0) {
          double y[4];
          stencil9<double>(c64, v64, gidx[j], P, y);
#pragma unroll
          for (int r = 0; r < 4; ++r) rr[j][r] = -y[r];
        }
    }
    __syncthreads();

    const double tol2 = p.tol * p.tol;
    int total_iters[4] = {0, 0, 0, 0};

    if (!MIXED) {
      // ================= plain FP64 CG ====================================
      double xr[NPT][4], qr[NPT][4];
#pragma unroll
      for (int j = 0; j < NPT; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          xr[j][r] = 0.0;
          qr[j][r] = 0.0;
        }
      if (warm) {
#pragma unroll
        for (int j = 0; j < NPT; ++j)
          if (gidx[j] >= 0) ld4(v64, gidx[j], xr[j]);
      }
      // v64 becomes p~ (zero on the boundary ring)
      for (int k = tid; k < 4 * N; k += NT) {
        int ix, iy;
        if (k < N) { ix = k; iy = 0; }
        else if (k < 2 * N) { ix = N; iy = k - N; }
        else if (k < 3 * N) { ix = N - (k - 2 * N); iy = N; }
        else { ix = 0; iy = N - (k - 3 * N); }
        const double z[4] = {0.0, 0.0, 0.0, 0.0};
        st4(v64, (iy + 1) * P + ix + 1, z);
      }
      double rho_p[8];
#pragma unroll
      for (int r = 0; r < 4; ++r) { rho_p[r] = 0.0; rho_p[4 + r] = 0.0; }
#pragma unroll
      for (int j = 0; j < NPT; ++j)
        if (gidx[j] >= 0) {
          st4(v64, gidx[j], rr[j]);
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            rho_p[r] = fma(rr[j][r], rr[j][r], rho_p[r]);
            rho_p[4 + r] = fma(rr[j][r] * dloc[j], rr[j][r], rho_p[4 + r]);
          }
        }
      warp_partials<8>(rho_p, red[0], warp, lane);
      __syncthreads();
      if (warp == 0) {
        const double t = warp0_finish<8>(red[0], NW, lane);
        const double nu = shfl_xor_d(t, 4);  // lane r (<4) gets value 4+r
        if (lane < 4) {
          cs.rho[lane] = t;
          const bool conv = nu <= tol2 * cs.bb[lane];
          cs.active[lane] = !conv;
          cs.iters[lane] = 0;
          cs.beta[lane] = 0.0;
        }
        __syncwarp();
        if (lane == 0) {
          int any = 0, nn2 = 0;
          for (int r = 0; r < 4; ++r) {
            any |= cs.active[r];
            if (cs.active[r] && cs.dmin * cs.rho[r] <= 100.0 * tol2 * cs.bb[r]) nn2 = 1;
          }
          cs.done = !any;
          cs.need_nu = nn2 || p.check_interval == 1;
        }
      }
      __syncthreads();
      int it = 0;
      while (!cs.done) {
        ++it;
        // q = A~ p, sigma = p.q
        double sg[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int j = 0; j < NPT; ++j)
          if (gidx[j] >= 0) {
            double pj[4];
            stencil9<double>(c64, v64, gidx[j], P, qr[j]);
            ld4(v64, gidx[j], pj);
#pragma unroll
            for (int r = 0; r < 4; ++r) sg[r] = fma(pj[r], qr[j][r], sg[r]);
          }
        warp_partials<4>(sg, red[1], warp, lane);
        __syncthreads();
        if (warp == 0) {
          const double t = warp0_finish<4>(red[1], NW, lane);
          if (lane < 4) {
            double a = 0.0;
            if (cs.active[lane]) {
              if (cs.rho[lane] == 0.0) {
                // exact solution reached in the previous step
                cs.active[lane] = 0;
                cs.iters[lane] = it - 1;
              } else {
                a = cs.rho[lane] / t;
                if (!isfinite(a) || !(t > 0.0)) {
                  a = 0.0;
                  cs.active[lane] = 0;
                  cs.iters[lane] = -it;  // breakdown marker
                }
              }
            }
            cs.alpha[lane] = a;
          }
        }
        __syncthreads();
        const bool need_nu = cs.need_nu;
        double al[4] = {cs.alpha[0], cs.alpha[1], cs.alpha[2], cs.alpha[3]};
        double rp[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) rp[r] = 0.0;
#pragma unroll
        for (int j = 0; j < NPT; ++j)
          if (gidx[j] >= 0) {
            double pj[4];
            ld4(v64, gidx[j], pj);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
              xr[j][r] = fma(al[r], pj[r], xr[j][r]);
              rr[j][r] = fma(-al[r], qr[j][r], rr[j][r]);
              rp[r] = fma(rr[j][r], rr[j][r], rp[r]);
            }
            if (need_nu) {
#pragma unroll
              for (int r = 0; r < 4; ++r) rp[4 + r] = fma(rr[j][r] * dloc[j], rr[j][r], rp[4 + r]);
            }
          }
        if (need_nu) {
          warp_partials<8>(rp, red[0], warp, lane);
        } else {
          double r4[4] = {rp[0], rp[1], rp[2], rp[3]};
          warp_partials<4>(r4, red[0], warp, lane);
        }
        __syncthreads();
        if (warp == 0) {
          double t, nu = 0.0;
          if (need_nu) {
            t = warp0_finish<8>(red[0], NW, lane);
            nu = shfl_xor_d(t, 4);
          } else {
            t = warp0_finish<4>(red[0], NW, lane);
          }
          if (lane < 4) {
            double b = 0.0;
            if (cs.active[lane]) {
              if (!isfinite(t)) {
                cs.active[lane] = 0;
                cs.iters[lane] = -it;
              } else if (t == 0.0 || (need_nu && nu <= tol2 * cs.bb[lane])) {
                cs.active[lane] = 0;
                cs.iters[lane] = it;
              } else if (it >= p.maxit) {
                cs.active[lane] = 0;
                cs.iters[lane] = -1000000 - it;  // maxit marker
              } else {
                b = t / cs.rho[lane];
                cs.rho[lane] = t;
              }
            }
            cs.beta[lane] = b;
          }
          __syncwarp();
          if (lane == 0) {
            int any = 0, nn2 = 0;
            for (int r = 0; r < 4; ++r) {
              any |= cs.active[r];
              if (cs.active[r] && cs.dmin * cs.rho[r] <= 100.0 * tol2 * cs.bb[r]) nn2 = 1;
            }
            cs.done = !any;
            cs.need_nu = nn2 || (p.check_interval > 0 && ((it + 1) % p.check_interval) == 0);
          }
        }
        __syncthreads();
        if (cs.done) break;
        const double be[4] = {cs.beta[0], cs.beta[1], cs.beta[2], cs.beta[3]};
#pragma unroll
        for (int j = 0; j < NPT; ++j)
          if (gidx[j] >= 0) {
            double pj[4];
            ld4(v64, gidx[j], pj);
#pragma unroll
            for (int r = 0; r < 4; ++r) pj[r] = fma(be[r], pj[r], rr[j][r]);
            st4(v64, gidx[j], pj);
          }
        __syncthreads();
      }
      // phi~ = [x~ ; D^1/2 g] into v64
#pragma unroll
      for (int j = 0; j < NPT; ++j)
        if (gidx[j] >= 0) st4(v64, gidx[j], xr[j]);
      for (int k = tid; k < 4 * N; k += NT) {
        int ix, iy;
        if (k < N) { ix = k; iy = 0; }
        else if (k < 2 * N) { ix = N; iy = k - N; }
        else if (k < 3 * N) { ix = N - (k - 2 * N); iy = N; }
        else { ix = 0; iy = N - (k - 3 * N); }
        const int g = (iy + 1) * P + ix + 1;
        double x[2], gv[4];
        bilinear_map(cs.corners, ix / (double)N, iy / (double)N, x);
        q1_eval<2>(cs.q1coef, cs.q1shift, cs.q1iscale, x, gv);
        const double sq = d64[g] * s64[g];
        double t[4] = {gv[0] * sq, gv[1] * sq, gv[2] * sq, gv[3] * sq};
        st4(v64, g, t);
      }
      __syncthreads();
      if (tid == 0) cs.refinements = 0;
    } else {
      // ================= MIXED: FP32 inner CG + FP64 refinement ===========
      // x~ lives in v64 (interior); r (FP64) in rr.  v32 holds p~ (FP32),
      // zero on the boundary ring.
      if (tid == 0) cs.refinements = 0;
      int ref = 0;
      for (;;) {
        // true residual norm and convergence test (FP64)
        double nup[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int j = 0; j < NPT; ++j)
          if (gidx[j] >= 0)
#pragma unroll
            for (int r = 0; r < 4; ++r) nup[r] = fma(rr[j][r] * dloc[j], rr[j][r], nup[r]);
        warp_partials<4>(nup, red[0], warp, lane);
        __syncthreads();
        if (warp == 0) {
          const double t = warp0_finish<4>(red[0], NW, lane);
          if (lane < 4) {
            if (!isfinite(t)) {
              cs.active[lane] = 0;
              cs.iters[lane] = -1;
            } else {
              cs.active[lane] = !(t <= tol2 * cs.bb[lane]);
            }
          }
          __syncwarp();
          if (lane == 0) {
            int any = 0;
            for (int r = 0; r < 4; ++r) any |= cs.active[r];
            if (any && ref >= p.max_refine) {
              for (int r = 0; r < 4; ++r)
                if (cs.active[r]) { cs.active[r] = 0; cs.iters[r] = -1000000; }
              any = 0;
            }
            cs.done = !any;
          }
        }
        __syncthreads();
        if (cs.done) break;
        ++ref;
        // ---- inner FP32 CG on A~ d = r (active RHS only)
        float act[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) act[r] = cs.active[r] ? 1.0f : 0.0f;
        float r32[NPT][4], d32[NPT][4], q32[NPT][4];
        float rho32[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int j = 0; j < NPT; ++j) {
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            r32[j][r] = (float)rr[j][r] * act[r];
            d32[j][r] = 0.0f;
            q32[j][r] = 0.0f;
          }
          if (gidx[j] >= 0) {
            st4(v32, gidx[j], r32[j]);
#pragma unroll
            for (int r = 0; r < 4; ++r) rho32[r] = fmaf(r32[j][r], r32[j][r], rho32[r]);
          }
        }
        // block reduce rho32 (all threads compute the totals redundantly)
        int buf = 0;
        {
          float tmp[4] = {rho32[0], rho32[1], rho32[2], rho32[3]};
          const float tot = warp_transpose_reduce<4>(tmp, lane);
          if ((lane & 7) == 0) red32[buf][warp * 4 + (lane >> 3)] = tot;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          float s = 0.f;
          for (int w = 0; w < NW; ++w) s += red32[buf][w * 4 + r];
          rho32[r] = s;
        }
        buf ^= 1;
        const float itol2 = p.inner_tol * p.inner_tol;
        float rho0[4] = {rho32[0], rho32[1], rho32[2], rho32[3]};
        bool inner_act[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) inner_act[r] = act[r] > 0.0f && rho32[r] > 0.0f;
        int iit = 0;
        for (;;) {
          bool any = inner_act[0] || inner_act[1] || inner_act[2] || inner_act[3];
          if (!any || iit >= p.inner_maxit) break;
          ++iit;
          // q = A~ p, sigma
          float sg[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
          for (int j = 0; j < NPT; ++j)
            if (gidx[j] >= 0) {
              float pj[4];
              stencil9<float>(c32, v32, gidx[j], P, q32[j]);
              ld4(v32, gidx[j], pj);
#pragma unroll
              for (int r = 0; r < 4; ++r) sg[r] = fmaf(pj[r], q32[j][r], sg[r]);
            }
          {
            const float tot = warp_transpose_reduce<4>(sg, lane);
            if ((lane & 7) == 0) red32[buf][warp * 4 + (lane >> 3)] = tot;
          }
          __syncthreads();
          float al[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            float s = 0.f;
            for (int w = 0; w < NW; ++w) s += red32[buf][w * 4 + r];
            al[r] = (inner_act[r] && s > 0.f) ? rho32[r] / s : 0.0f;
          }
          buf ^= 1;
          float rp[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
          for (int j = 0; j < NPT; ++j)
            if (gidx[j] >= 0) {
              float pj[4];
              ld4(v32, gidx[j], pj);
#pragma unroll
              for (int r = 0; r < 4; ++r) {
                d32[j][r] = fmaf(al[r], pj[r], d32[j][r]);
                r32[j][r] = fmaf(-al[r], q32[j][r], r32[j][r]);
                rp[r] = fmaf(r32[j][r], r32[j][r], rp[r]);
              }
            }
          {
            const float tot = warp_transpose_reduce<4>(rp, lane);
            if ((lane & 7) == 0) red32[buf][warp * 4 + (lane >> 3)] = tot;
          }
          __syncthreads();
          float be[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            float s = 0.f;
            for (int w = 0; w < NW; ++w) s += red32[buf][w * 4 + r];
            be[r] = 0.0f;
            if (inner_act[r]) {
              if (!(s <= itol2 * rho0[r]) && isfinite(s)) {
                be[r] = s / rho32[r];
                rho32[r] = s;
              } else {
                inner_act[r] = false;
              }
              total_iters[r] += 1;
            }
          }
          buf ^= 1;
#pragma unroll
          for (int j = 0; j < NPT; ++j)
            if (gidx[j] >= 0) {
              float pj[4];
              ld4(v32, gidx[j], pj);
#pragma unroll
              for (int r = 0; r < 4; ++r) pj[r] = fmaf(be[r], pj[r], r32[j][r]);
              st4(v32, gidx[j], pj);
            }
          __syncthreads();
        }
        // ---- x~ += d (FP64), new FP64 residual r = -(A~ phi~)_I
#pragma unroll
        for (int j = 0; j < NPT; ++j)
          if (gidx[j] >= 0) {
            double xj[4];
            ld4(v64, gidx[j], xj);
#pragma unroll
            for (int r = 0; r < 4; ++r) xj[r] += (double)d32[j][r];
            st4(v64, gidx[j], xj);
          }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < NPT; ++j)
          if (gidx[j] >= 0) {
            double y[4];
            stencil9<double>(c64, v64, gidx[j], P, y);
#pragma unroll
            for (int r = 0; r < 4; ++r) rr[j][r] = -y[r];
          }
      }
      if (tid == 0) cs.refinements = ref;
      __syncthreads();
    }

    // ---------------- epilogue: M, F, true residual ----------------------
    {
      double acc[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) acc[i] = 0.0;
      for (int k = tid; k < n * n; k += NT) {
        const int ix = k % n, iy = k / n;
        const int g = (iy + 1) * P + ix + 1;
        double y[4], ph[4];
        stencil9<double>(c64, v64, g, P, y);
        ld4(v64, g, ph);
        const double bl = b64[g];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[4 * i + j] = fma(ph[i], y[j], acc[4 * i + j]);
          acc[16 + i] = fma(ph[i], bl, acc[16 + i]);
        }
        if (ix > 0 && iy > 0 && ix < N && iy < N) {
          const double d = d64[g];
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[20 + j] = fma(y[j] * d, y[j], acc[20 + j]);
        }
        if (p.basis) {
          const double s = s64[g];
          double *out = p.basis + (p.basis_offset ? p.basis_offset[cell] : (int64_t)cell * 4 * n * n);
#pragma unroll
          for (int i = 0; i < 4; ++i) out[(int64_t)i * n * n + k] = ph[i] * s;
        }
      }
      const double tot = warp_transpose_reduce<32>(acc, lane);
      red[0][warp * 32 + lane] = tot;
      __syncthreads();
      if (warp == 0) {
        double s = 0.0;
        for (int w = 0; w < NW; ++w) s += red[0][w * 32 + lane];
        // lane v holds value v
        if (lane < 16) p.M[(int64_t)cell * 16 + lane] = s;
        else if (lane < 20) p.F[(int64_t)cell * 4 + (lane - 16)] = s;
        double rel = 0.0;
        if (lane >= 20 && lane < 24) {
          const double bb = cs.bb[lane - 20];
          rel = bb > 0.0 ? sqrt(s / bb) : sqrt(s);
        }
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) rel = fmax(rel, shfl_xor_d(rel, m));
        if (lane < 4) {
          int itv = cs.iters[lane];
          if (MIXED) {
            // iters holds -1 / -1000000 markers only; count inner iterations
            if (p.iters) p.iters[(int64_t)cell * 4 + lane] = total_iters[lane];
          } else if (p.iters) {
            p.iters[(int64_t)cell * 4 + lane] = itv >= 0 ? itv : (itv <= -1000000 ? -itv - 1000000 : -itv);
          }
        }
        if (lane == 0) {
          int st = cs.status;  // MSFEM_CELL_NAN when a diagonal was not positive
          for (int r = 0; r < 4; ++r) {
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
      __syncthreads();
    }
  }
}

}  // namespace msfem
