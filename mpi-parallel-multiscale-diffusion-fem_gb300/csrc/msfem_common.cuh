// msfem_common.cuh -- device-side building blocks shared by the 2D and 3D
// multiscale-basis kernels: kernel parameter block, block reductions,
// coefficient evaluation at Gauss points and the coarse Q1 (BasisQ1)
// interpolation data.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "msfem_gpu.h"

namespace msfem {

// Parameters of one batch launch (all pointers are device pointers).
struct KernelParams {
  int dim;
  int n_cells;
  int n_fine_uniform;
  const double *corners;       // [cell][2^d][d]
  const int32_t *n_fine;       // [cell] or nullptr
  const int32_t *order;        // work queue: cell ids in processing order
  unsigned int *queue;         // work-queue head (zeroed before the launch)
  int coef_kind;               // CONSTANT / REFERENCE / SINSIN / TABULATED
  int ncomp;
  double cparams[8];           // kind-specific, pre-processed on the host
  const double *qp_values;
  const int64_t *qp_offset;    // nullptr = uniform cell blocks
  double f_value;
  const double *f_qp;          // f at the Gauss points [q][fine cell] per cell, nullptr = f_value
  const int64_t *f_qp_offset;  // nullptr = uniform cell blocks of 2^d N^d
  double tol;                  // residual tolerance (relative, or absolute with tol_abs)
  int tol_abs;                 // 1: stop at ||r|| <= tol, 0: at ||r|| <= tol ||b||
  int maxit;
  int check_interval;          // 0 = adaptive
  const double *warm_basis;    // nullptr = cold start
  const int64_t *basis_offset; // [cell] offset of the cell's basis block (uneven N)
  double *M;
  double *F;
  double *basis;               // nullptr = not requested
  int32_t *status;
  int32_t *iters;              // [cell][2^d]
  double *rel_res;             // [cell] max true relative residual over the 2^d solves
  int32_t *refinements;        // [cell] mixed: outer FP64 refinement steps
  float inner_tol;             // mixed: inner FP32 relative reduction
  int inner_maxit;             // mixed: inner iteration cap per refinement
  int max_refine;              // mixed: outer refinement cap
  float cheb_ratio;            // mixed, polynomial-preconditioned: b / a of the Chebyshev interval
};

// The reference's pi constant (include/coefficients/coefficients.h:21).
constexpr double kPiD = 3.14592653509793218403;

__device__ __forceinline__ double shfl_xor_d(double v, int m) {
  return __shfl_xor_sync(0xffffffffu, v, m);
}
__device__ __forceinline__ float shfl_xor_d(float v, int m) {
  return __shfl_xor_sync(0xffffffffu, v, m);
}

// Transpose-reduce of K values across a warp (K a power of two <= 32).  On
// return lane l holds the warp total of value index  (l >> (5 - log2 K)),
// i.e. value v sits in lanes [v * 32/K, (v+1) * 32/K).  Each halving step
// sends half of the remaining values to the partner lane, so the adds per
// lane are K/2 + K/4 + ... + 1 + (5 - log2 K) instead of 5 K.
template <int K, typename T>
__device__ __forceinline__ T warp_transpose_reduce(T (&v)[K], int lane) {
  static_assert(K >= 1 && K <= 32 && (K & (K - 1)) == 0, "K power of two");
  constexpr int LOGK = (K >= 32) ? 5 : (K >= 16) ? 4 : (K >= 8) ? 3 : (K >= 4) ? 2 : (K >= 2) ? 1 : 0;
  // Level l (mask 16 >> l) halves the live set. Values live in v[0..cnt).
#pragma unroll
  for (int l = 0; l < LOGK; ++l) {
    const int mask = 16 >> l;
    const int half = K >> (l + 1);
    const bool upper = (lane & mask) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      T keep = upper ? v[i + half] : v[i];
      T send = upper ? v[i] : v[i + half];
      v[i] = keep + shfl_xor_d(send, mask);
    }
  }
  T s = v[0];
#pragma unroll
  for (int m = 16 >> LOGK; m >= 1; m >>= 1) s += shfl_xor_d(s, m);
  return s;
}

// Warp 0 finishes a K-value block reduction: red holds NW*K warp partials
// ([warp][value]); on return lane l holds the block total of value l % K.
template <int K, typename T>
__device__ __forceinline__ T warp_finish(const T *red, int NW, int lane) {
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

// QGauss(2) point i in [0,1] (reference coordinate of the two-point rule).
__device__ __forceinline__ double gauss2(int i) {
  return i ? 0.78867513459481288225457439025098 : 0.21132486540518711774542560974902;
}

// Lane that holds value index `vi` of a K-value transpose-reduce.
template <int K>
__device__ __forceinline__ int transpose_reduce_lane(int vi) { return vi * (32 / K); }

// ---------------------------------------------------------------------------
// Coarse Q1 nodal functions (Coefficients::BasisQ1, basis_q1.tpp:26-158).
// The 2^d polynomials in span{1,x,y,xy} (2D) / span{1,x,y,z,xy,yz,xz,xyz} (3D)
// interpolating the coarse vertices.  Built in the translated, scaled
// coordinates x' = (x - v0)/H, which span the same space (hence the same
// interpolant) with a well-conditioned Vandermonde matrix.  coef[m*nv + i]:
// coefficient of monomial m in basis function i.
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void q1_monomials(const double *xp, double *m) {
  if (DIM == 2) {
    m[0] = 1.0; m[1] = xp[0]; m[2] = xp[1]; m[3] = xp[0] * xp[1];
  } else {
    m[0] = 1.0; m[1] = xp[0]; m[2] = xp[1]; m[3] = xp[2];
    m[4] = xp[0] * xp[1]; m[5] = xp[1] * xp[2]; m[6] = xp[0] * xp[2];
    m[7] = xp[0] * xp[1] * xp[2];
  }
}

// Single-thread Gauss-Jordan inverse of the nv x nv Vandermonde matrix.
// Returns false for a singular (degenerate) cell.
template <int DIM>
__device__ bool q1_setup(const double *corners, double *coef, double *shift,
                         double *inv_scale) {
  constexpr int NV = 1 << DIM;
  double H = 0.0;
  for (int a = 0; a < DIM; ++a) shift[a] = corners[a];
  for (int v = 1; v < NV; ++v)
    for (int a = 0; a < DIM; ++a) H = fmax(H, fabs(corners[v * DIM + a] - corners[a]));
  if (!(H > 0.0)) return false;
  const double ih = 1.0 / H;
  *inv_scale = ih;
  double w[NV][2 * NV];
  for (int v = 0; v < NV; ++v) {
    double xp[3], m[8];
    for (int a = 0; a < DIM; ++a) xp[a] = (corners[v * DIM + a] - shift[a]) * ih;
    q1_monomials<DIM>(xp, m);
    for (int j = 0; j < NV; ++j) {
      w[v][j] = m[j];
      w[v][NV + j] = (j == v) ? 1.0 : 0.0;
    }
  }
  for (int col = 0; col < NV; ++col) {
    int piv = col;
    for (int r = col + 1; r < NV; ++r)
      if (fabs(w[r][col]) > fabs(w[piv][col])) piv = r;
    if (w[piv][col] == 0.0) return false;
    if (piv != col)
      for (int j = 0; j < 2 * NV; ++j) {
        double t = w[col][j]; w[col][j] = w[piv][j]; w[piv][j] = t;
      }
    const double id = 1.0 / w[col][col];
    for (int j = 0; j < 2 * NV; ++j) w[col][j] *= id;
    for (int r = 0; r < NV; ++r) {
      if (r == col) continue;
      const double f = w[r][col];
      if (f != 0.0)
        for (int j = 0; j < 2 * NV; ++j) w[r][j] -= f * w[col][j];
    }
  }
  // inverse(P)[m][i]: row m = monomial, column i = vertex/basis index
  for (int m = 0; m < NV; ++m)
    for (int i = 0; i < NV; ++i) coef[m * NV + i] = w[m][NV + i];
  return true;
}

template <int DIM>
__device__ __forceinline__ void q1_eval(const double *coef, const double *shift,
                                        double inv_scale, const double *x,
                                        double *out) {
  constexpr int NV = 1 << DIM;
  double xp[3], m[8];
  for (int a = 0; a < DIM; ++a) xp[a] = (x[a] - shift[a]) * inv_scale;
  q1_monomials<DIM>(xp, m);
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NV; ++k) s = fma(coef[k * NV + i], m[k], s);
    out[i] = s;
  }
}

// ---------------------------------------------------------------------------
// Coefficient at a Gauss point, as the symmetric tensor components
// (a11, a12, a22) in 2D or (a11, a12, a13, a22, a23, a33) in 3D.
//   CONSTANT  : cparams[0..]
//   REFERENCE : c(x) * (R R^T) with R R^T pre-multiplied on the host
//               (MatrixCoeff::value_list, matrix_coeff.tpp:66-91)
//   SINSIN    : 1 + amp sin(2 pi x/eps) sin(2 pi y/eps) [sin(2 pi z/eps)]
//   TABULATED : loaded from qp_values (layout [comp][q][fine cell])
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void coef_at(const KernelParams &p, const double *xq,
                                        const double *__restrict__ tab, int q,
                                        int nfc, int fc, double *A) {
  constexpr int NC = DIM == 2 ? 3 : 6;
  constexpr int NQ = 1 << DIM;
  switch (p.coef_kind) {
  case MSFEM_COEF_CONSTANT:
#pragma unroll
    for (int k = 0; k < NC; ++k) A[k] = p.cparams[k];
    break;
  case MSFEM_COEF_REFERENCE: {
    // 1 - 0.9999 (0.5 sin(2 PI_D 57 x) + 0.5 sin(2 PI_D 57 y))
    const double c = 1.0 * (1.0 - 0.9999 * (0.5 * sin(2 * kPiD * 57 * xq[0]) +
                                            0.5 * sin(2 * kPiD * 57 * xq[1])));
#pragma unroll
    for (int k = 0; k < NC; ++k) A[k] = c * p.cparams[k];
    break;
  }
  case MSFEM_COEF_SINSIN: {
    const double ie = 2.0 / p.cparams[1];
    double s = sinpi(xq[0] * ie) * sinpi(xq[1] * ie);
    if (DIM == 3) s *= sinpi(xq[2] * ie);
    const double a = 1.0 + p.cparams[0] * s;
#pragma unroll
    for (int k = 0; k < NC; ++k) A[k] = 0.0;
    A[0] = a;
    if (DIM == 2) A[2] = a; else { A[3] = a; A[5] = a; }
    break;
  }
  default: {  // TABULATED
    if (p.ncomp == 1) {
      const double a = __ldg(tab + (int64_t)q * nfc + fc);
#pragma unroll
      for (int k = 0; k < NC; ++k) A[k] = 0.0;
      A[0] = a;
      if (DIM == 2) A[2] = a; else { A[3] = a; A[5] = a; }
    } else {
#pragma unroll
      for (int k = 0; k < NC; ++k) A[k] = __ldg(tab + ((int64_t)k * NQ + q) * nfc + fc);
    }
    break;
  }
  }
}

}  // namespace msfem
