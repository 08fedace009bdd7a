// msfem_kernel2d.cuh -- 2D multiscale-basis kernels for sm_103a.
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
//      M_ij = phi~_i^T A~ phi~_j,  phi~ = D^1/2 phi,  F_i = phi~_i^T D^-1/2 b.
//
// Kernels:
//   msfem2d_kernel        plain FP64 CG (the drop-in form); bound by the FP64 pipe.
//   msfem2d_mixed_kernel  FP64 outer loop r = b - A x (true FP64 residual),
//                         inner FP32 CG on A~ d = r, x += d in FP64.  Threads
//                         own vertical strips of S nodes (register blocking).
//
// Shared-memory layout (node-major, 4 values per node; P = N + 3: the
// (N+1)^2 node grid plus a zero ring, node (ix,iy) at (iy+1) P + ix + 1):
//   c64 [G][4]  scaled couplings E, NE, N, NW of each node (FP64)
//   v64 [G][4]  FP64 work vector of the 4 RHS (p~ in FP64 CG, phi~ otherwise)
//   d64 [G]     diagonal D (D^-1/2 is recomputed where needed)
//   v32 [G][4]  FP32 search direction of the mixed inner loop
//   v32b[G][4]  FP32 second exchange buffer (polynomial-preconditioned form)
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
  static constexpr size_t kD64 = al(kV64 + sizeof(double) * 4 * G);
  static constexpr size_t kEndFP64 = al(kD64 + sizeof(double) * G);
  static constexpr size_t kV32 = kEndFP64;
  static constexpr size_t kEndMixed = al(kV32 + sizeof(float) * 4 * G);
  static constexpr size_t kV32B = kEndMixed;  // second FP32 exchange buffer (polynomial preconditioner)
  static constexpr size_t kEndCheb = al(kV32B + sizeof(float) * 4 * G);
  static constexpr size_t bytes(bool mixed) { return mixed ? kEndMixed : kEndFP64; }
  static_assert(kV64 % 16 == 0 && kV32 % 16 == 0, "vector alignment");
};

// Coarse-grid arrays of the two-level preconditioner (mixed form), after the
// second FP32 exchange buffer.  Coarse spacing CH fine cells, so at most
// NC = NMAX / CH coarse intervals and NI = (NC - 1)^2 interior coarse nodes:
//   ub  [2][NC][33] float4  row-block partial restrictions onto the lower /
//                           upper coarse row, by fine column (rows of 33: the
//                           per-coarse-node column sums read distinct banks);
//                           during the set-up the band Cholesky factor of Ac
//   rc  [NI] float4         restricted residual, 4 RHS
//   ec  [NC+1][NC+1] float4 coarse correction with a zero boundary ring
//   a0  [NI][NI] float      set-up scratch: row j = column j of L^-1 (Ac = L L^T)
//   a1  [NI][NI] float      the Galerkin coarse matrix Ac, then Ac^-1 = L^-T L^-1
template <int NMAX, int CH>
struct Coarse2D {
  using L = Smem2D<NMAX>;
  static constexpr int NC = CH > 0 ? NMAX / CH : 2;
  static constexpr int NI = (NC - 1) * (NC - 1);
  static constexpr size_t kUB = L::kEndCheb;
  static constexpr size_t kRC = L::al(kUB + 16 * 2 * 33 * NC);
  static constexpr size_t kEC = L::al(kRC + 16 * NI);
  static constexpr size_t kA0 = L::al(kEC + 16 * (NC + 1) * (NC + 1));
  static constexpr size_t kA1 = L::al(kA0 + sizeof(float) * NI * NI);
  static constexpr size_t kEnd = L::al(kA1 + sizeof(float) * NI * NI);
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

// FP32 -> FP64 conversion by the IEEE-754 bit layouts, on the integer pipe
// (measured cheaper than the conversion instruction in the mixed kernel's
// FP64 update).  Exact for normal numbers and zeros; FP32 subnormals become
// signed zeros, inf/NaN stay inf/NaN.
__device__ __forceinline__ double f32_to_f64(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint32_t hi_sign = u & 0x80000000u;
  const uint32_t m = u & 0x7FFFFFu;
  uint32_t hi, lo;
  if (e == 0u) {
    hi = hi_sign;
    lo = 0u;
  } else {
    const uint32_t ed = e == 0xFFu ? 0x7FFu : e + (1023u - 127u);
    hi = hi_sign | (ed << 20) | (m >> 3);
    lo = m << 29;
  }
  return __hiloint2double((int)hi, (int)lo);
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

// y = A v at node g with the unscaled operator: diagonal d[g] and the 8
// couplings of c (as stencil9), 4 RHS.
__device__ __forceinline__ void stencil9_unscaled(const double *__restrict__ c, const double *__restrict__ d,
                                                  const double *__restrict__ v, int g, int P, double (&y)[4]) {
  double cc[4], t[4];
  ld4(c, g, cc);
  const double cW = c[4 * (g - 1) + 0];
  const double cS = c[4 * (g - P) + 2];
  const double cSW = c[4 * (g - P - 1) + 1];
  const double cSE = c[4 * (g - P + 1) + 3];
  const double dg = d[g];
  ld4(v, g, y);
#pragma unroll
  for (int r = 0; r < 4; ++r) y[r] *= dg;
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

// Block-uniform scalars of one cell, in shared memory.
struct CellShared2D {
  double corners[8];
  double q1coef[16];
  double q1shift[2];
  double q1iscale;
  double jinv_g[9];   // affine cells: (a11,a12,a22) -> w|det| Jinv A Jinv^T as (G11,G12,G22)
  double jfine[4];    // affine cells: fine-cell Jacobian, columns dx/dxi, dx/deta
  double absdet;      // affine cells: |det J_fine|
  double bb[4];       // ||b_i||^2 (unscaled)
  double bthr[4];     // stopping scale: ||b_i||^2 (relative tolerance) or 1 (absolute)
  double nu[4];       // last ||r_i||^2 (unscaled)
  double rho[4];
  double alpha[4];
  double beta[4];
  double dmin;
  int active[4];
  int iters[4];
  int status;
  int affine;
  int axis;           // affine cell with axis-aligned edges: G = diag(jinv_g[0], jinv_g[4], jinv_g[8]) A
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
// l_b(gauss2(qb)),  l_0(t) = 1 - t,  l_1(t) = t
__device__ __forceinline__ double lval(int b, int qb) {
  return b ? gauss2(qb) : gauss2(1 - qb);
}

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000ll); }

// Boundary node k in [0, 4N): walk around the cell boundary.
__device__ __forceinline__ void boundary_node(int k, int N, int &ix, int &iy) {
  if (k < N) { ix = k; iy = 0; }
  else if (k < 2 * N) { ix = N; iy = k - N; }
  else if (k < 3 * N) { ix = N - (k - 2 * N); iy = N; }
  else { ix = 0; iy = N - (k - 3 * N); }
}

// BasisQ1 data of a 2D cell (the q1_setup<2> interpolant) in closed form.
// In the translated, scaled coordinates x' = (x - v0) / H vertex 0 sits at
// the origin, so the Vandermonde row of vertex 0 is (1, 0, 0, 0): the
// constant coefficient of basis i is delta_i0, and the other three solve
// Q c = (delta_iv - delta_i0)_{v=1..3} with Q's rows (a_v, b_v, a_v b_v),
// (a_v, b_v) = x'_v.  Q^-1 = adj(Q) / det(Q).  A single thread runs this
// (about 70 FP64 operations instead of a pivoted elimination on a 4 x 8
// array).  Returns false for a degenerate cell.
__device__ inline bool q1_setup2d_closed(const double *cr, double *coef, double *shift, double *inv_scale) {
  shift[0] = cr[0];
  shift[1] = cr[1];
  double H = 0.0;
#pragma unroll
  for (int v = 1; v < 4; ++v) H = fmax(H, fmax(fabs(cr[2 * v] - cr[0]), fabs(cr[2 * v + 1] - cr[1])));
  if (!(H > 0.0)) return false;
  const double ih = 1.0 / H;
  *inv_scale = ih;
  double a[3], b[3], e[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    a[v] = (cr[2 * (v + 1)] - cr[0]) * ih;
    b[v] = (cr[2 * (v + 1) + 1] - cr[1]) * ih;
    e[v] = a[v] * b[v];
  }
  // cofactors C[v][m] of Q (v: vertex row 1..3, m: monomial x', y', x'y')
  double C[3][3];
  C[0][0] = b[1] * e[2] - e[1] * b[2];
  C[0][1] = e[1] * a[2] - a[1] * e[2];
  C[0][2] = a[1] * b[2] - b[1] * a[2];
  C[1][0] = e[0] * b[2] - b[0] * e[2];
  C[1][1] = a[0] * e[2] - e[0] * a[2];
  C[1][2] = b[0] * a[2] - a[0] * b[2];
  C[2][0] = b[0] * e[1] - e[0] * b[1];
  C[2][1] = e[0] * a[1] - a[0] * e[1];
  C[2][2] = a[0] * b[1] - b[0] * a[1];
  const double det = a[0] * C[0][0] + b[0] * C[0][1] + e[0] * C[0][2];
  if (!(fabs(det) > 0.0) || !isfinite(det)) return false;
  const double idet = 1.0 / det;
  coef[0] = 1.0;
  coef[1] = coef[2] = coef[3] = 0.0;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    double s = 0.0;
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      const double q = C[v][m] * idet;  // (Q^-1)[m][v]
      coef[(m + 1) * 4 + v + 1] = q;
      s += q;
    }
    coef[(m + 1) * 4] = -s;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Shared per-cell phases
// ---------------------------------------------------------------------------

// Geometry and Q1 data of one cell (corners, BasisQ1 coefficients, the
// affine-cell Jacobian data).  Returns the cell status.
template <int NMAX>
__device__ int cell_geometry2d(const KernelParams &p, CellShared2D &cs, int cell, int N, int tid) {
  if (tid < 8) cs.corners[tid] = p.corners[(int64_t)cell * 8 + tid];
  __syncthreads();
  if (tid == 0) {
    const double *cr = cs.corners;
    int st = MSFEM_CELL_CONVERGED;
    if (N < 1 || N > NMAX) st = MSFEM_CELL_BAD_INPUT;
    if (st == MSFEM_CELL_CONVERGED && !q1_setup2d_closed(cr, cs.q1coef, cs.q1shift, &cs.q1iscale))
      st = MSFEM_CELL_BAD_INPUT;
    // parallelogram test v0 + v3 == v1 + v2 (exact)
    const int aff = (cr[0] + cr[6] == cr[2] + cr[4]) && (cr[1] + cr[7] == cr[3] + cr[5]);
    cs.affine = aff;
    cs.axis = aff && cr[3] == cr[1] && cr[4] == cr[0];
    cs.refinements = 0;
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
  return cs.status;
}

// Geometry, Q1 data, zeroed arrays.  Returns the cell status.
template <int NMAX, int NT>
__device__ int cell_begin(const KernelParams &p, CellShared2D &cs, int cell, int N,
                          double *c64, double *v64, double *d64, float *v32, int tid) {
  const int P = N + 3, G = P * P;
  // 16-byte stores (every array starts on a 128-byte boundary)
  const double2 z2 = make_double2(0.0, 0.0);
  for (int i = tid; i < 2 * G; i += NT) {
    reinterpret_cast<double2 *>(c64)[i] = z2;
    reinterpret_cast<double2 *>(v64)[i] = z2;
  }
  for (int i = tid; i < (G + 1) / 2; i += NT) reinterpret_cast<double2 *>(d64)[i] = z2;
  if (v32)
    for (int i = tid; i < G; i += NT) reinterpret_cast<float4 *>(v32)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tid < 4) { cs.iters[tid] = 0; cs.active[tid] = 1; cs.nu[tid] = 0.0; }
  return cell_geometry2d<NMAX>(p, cs, cell, N, tid);
}

// Malformed cell: NaN outputs and the status word, then move on.
__device__ inline void cell_report_bad(const KernelParams &p, const CellShared2D &cs, int cell, int tid) {
  if (tid < 16) p.M[(int64_t)cell * 16 + tid] = qnan();
  if (tid < 4) {
    p.F[(int64_t)cell * 4 + tid] = qnan();
    if (p.iters) p.iters[(int64_t)cell * 4 + tid] = 0;
  }
  if (tid == 0) {
    p.status[cell] = cs.status;
    if (p.rel_res) p.rel_res[cell] = qnan();
    if (p.refinements) p.refinements[cell] = 0;
  }
}

// QGauss(2) element matrix of fine cell (cx, cy): diagonal Kd[4] and the
// six couplings Ko = (K01, K02, K03, K12, K13, K23).  Returns false for an
// inverted fine cell.
__device__ __forceinline__ bool element2d(const KernelParams &p, const CellShared2D &cs,
                                          const double *__restrict__ tab, int N, int cx, int cy,
                                          bool need_x, double (&Kd)[4], double (&Ko)[6]) {
  const int nfc = N * N, fc = cx + N * cy;
  if (cs.affine) {
    // G_q = w|det| Jinv A_q Jinv^T, then moments of the tensor-product Q1
    // gradients: d psi/d xi depends on eta only and d psi/d eta on xi only.
    double G11[4], G12[4], G22[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      double xq[2] = {0.0, 0.0}, A[3];
      if (need_x) {
        const double u = cx + gauss2(q & 1), v = cy + gauss2(q >> 1);
        xq[0] = cs.corners[0] + cs.jfine[0] * u + cs.jfine[2] * v;
        xq[1] = cs.corners[1] + cs.jfine[1] * u + cs.jfine[3] * v;
      }
      coef_at<2>(p, xq, tab, q, nfc, fc, A);
      if (cs.axis) {
        // the other six entries of jinv_g are zero: the same sums, 3 products
        G11[q] = cs.jinv_g[0] * A[0];
        G12[q] = cs.jinv_g[4] * A[1];
        G22[q] = cs.jinv_g[8] * A[2];
      } else {
        G11[q] = cs.jinv_g[0] * A[0] + cs.jinv_g[1] * A[1] + cs.jinv_g[2] * A[2];
        G12[q] = cs.jinv_g[3] * A[0] + cs.jinv_g[4] * A[1] + cs.jinv_g[5] * A[2];
        G22[q] = cs.jinv_g[6] * A[0] + cs.jinv_g[7] * A[1] + cs.jinv_g[8] * A[2];
      }
    }
    const double Ay[2] = {G11[0] + G11[1], G11[2] + G11[3]};  // sum over qx
    const double Bx[2] = {G22[0] + G22[2], G22[1] + G22[3]};  // sum over qy
    double Pyy[2][2], Pxx[2][2], Q[2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        Pyy[a][b] = Ay[0] * (lval(a, 0) * lval(b, 0)) + Ay[1] * (lval(a, 1) * lval(b, 1));
        Pxx[a][b] = Bx[0] * (lval(a, 0) * lval(b, 0)) + Bx[1] * (lval(a, 1) * lval(b, 1));
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q) s = fma(G12[q], lval(a, q >> 1) * lval(b, q & 1), s);
        Q[a][b] = s;  // a: y-index (of eta), b: x-index (of xi)
      }
    auto Kij = [&](int i, int j) {
      const int ix = i & 1, iy = i >> 1, jx = j & 1, jy = j >> 1;
      const double sxi = ix ? 1.0 : -1.0, syi = iy ? 1.0 : -1.0;
      const double sxj = jx ? 1.0 : -1.0, syj = jy ? 1.0 : -1.0;
      return (sxi * sxj) * Pyy[iy][jy] + (syi * syj) * Pxx[ix][jx] + (sxi * syj) * Q[iy][jx] +
             (syi * sxj) * Q[jy][ix];
    };
#pragma unroll
    for (int i = 0; i < 4; ++i) Kd[i] = Kij(i, i);
    Ko[0] = Kij(0, 1); Ko[1] = Kij(0, 2); Ko[2] = Kij(0, 3);
    Ko[3] = Kij(1, 2); Ko[4] = Kij(1, 3); Ko[5] = Kij(2, 3);
    return true;
  }
  // general bilinear cell: per-Gauss-point Jacobian
  const double invN = 1.0 / (double)N;
  double V[8];
  bilinear_map(cs.corners, cx * invN, cy * invN, V + 0);
  bilinear_map(cs.corners, (cx + 1) * invN, cy * invN, V + 2);
  bilinear_map(cs.corners, cx * invN, (cy + 1) * invN, V + 4);
  bilinear_map(cs.corners, (cx + 1) * invN, (cy + 1) * invN, V + 6);
  double K[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) K[i][j] = 0.0;
  bool ok = true;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int qx = q & 1, qy = q >> 1;
    double J00 = 0, J01 = 0, J10 = 0, J11 = 0, xq[2] = {0.0, 0.0};
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
    if (!(det > 0.0)) ok = false;
    const double id = 1.0 / det;
    const double i00 = J11 * id, i01 = -J01 * id, i10 = -J10 * id, i11 = J00 * id;
    const double w = 0.25 * fabs(det);
    double A[3];
    coef_at<2>(p, xq, tab, q, nfc, fc, A);
    const double t00 = i00 * A[0] + i01 * A[1], t01 = i00 * A[1] + i01 * A[2];
    const double t10 = i10 * A[0] + i11 * A[1], t11 = i10 * A[1] + i11 * A[2];
    const double Gm0 = w * (t00 * i00 + t01 * i01);
    const double Gm1 = w * (t00 * i10 + t01 * i11);
    const double Gm2 = w * (t10 * i10 + t11 * i11);
    double gx[4], gy[4], ax[4], ay[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int kx = k & 1, ky = k >> 1;
      gx[k] = (kx ? 1.0 : -1.0) * lval(ky, qy);
      gy[k] = (ky ? 1.0 : -1.0) * lval(kx, qx);
      ax[k] = Gm0 * gx[k] + Gm1 * gy[k];
      ay[k] = Gm1 * gx[k] + Gm2 * gy[k];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = i; j < 4; ++j) K[i][j] = fma(gx[i], ax[j], fma(gy[i], ay[j], K[i][j]));
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) Kd[i] = K[i][i];
  Ko[0] = K[0][1]; Ko[1] = K[0][2]; Ko[2] = K[0][3];
  Ko[3] = K[1][2]; Ko[4] = K[1][3]; Ko[5] = K[2][3];
  return ok;
}

// Assembly: 4-colour scatter of the element matrices into the node stencil.
// NODIAG: the element diagonals are not formed; every node's diagonal is
// minus the sum of its 8 couplings afterwards (Q1 element matrices have zero
// row sums: constants lie in the kernel of the gradient), which saves FP64
// work per element at the price of 7 additions per node.
template <int NT, bool NODIAG = false>
__device__ void assemble2d(const KernelParams &p, CellShared2D &cs, int cell, int N,
                           double *c64, double *d64, int tid) {
  const int P = N + 3, nfc = N * N;
  const double *tab = nullptr;
  if (p.coef_kind == MSFEM_COEF_TABULATED)
    tab = p.qp_values + (p.qp_offset ? p.qp_offset[cell] : (int64_t)cell * p.ncomp * 4 * nfc);
  const bool need_x = p.coef_kind != MSFEM_COEF_TABULATED && p.coef_kind != MSFEM_COEF_CONSTANT;
  for (int col = 0; col < 4; ++col) {
    const int ox = col & 1, oy = col >> 1;
    const int nx = (N - ox + 1) >> 1, ny = (N - oy + 1) >> 1;
    for (int idx = tid; idx < nx * ny; idx += NT) {
      const int cx = ox + 2 * (idx % nx), cy = oy + 2 * (idx / nx);
      double Kd[4], Ko[6];
      if (!element2d(p, cs, tab, N, cx, cy, need_x, Kd, Ko)) cs.status = MSFEM_CELL_BAD_INPUT;
      const int g0 = (cy + 1) * P + cx + 1;
      const int g1 = g0 + 1, g2 = g0 + P, g3 = g0 + P + 1;
      if (!NODIAG) { d64[g0] += Kd[0]; d64[g1] += Kd[1]; d64[g2] += Kd[2]; d64[g3] += Kd[3]; }
      c64[4 * g0 + 0] += Ko[0];  // E  of node 0 (0-1)
      c64[4 * g2 + 0] += Ko[5];  // E  of node 2 (2-3)
      c64[4 * g0 + 2] += Ko[1];  // N  of node 0 (0-2)
      c64[4 * g1 + 2] += Ko[4];  // N  of node 1 (1-3)
      c64[4 * g0 + 1] += Ko[2];  // NE of node 0 (0-3)
      c64[4 * g1 + 3] += Ko[3];  // NW of node 1 (1-2)
    }
    __syncthreads();
  }
  if constexpr (NODIAG) {
    const int n = N + 1;
    for (int k = tid; k < n * n; k += NT) {
      const int g = (k / n + 1) * P + k % n + 1;
      double cc[4];
      ld4(c64, g, cc);
      d64[g] = -(((cc[0] + cc[1]) + (cc[2] + cc[3])) +
                 ((c64[4 * (g - 1) + 0] + c64[4 * (g - P) + 2]) +
                  (c64[4 * (g - P - 1) + 1] + c64[4 * (g - P + 1) + 3])));
    }
    __syncthreads();
  }
}

// Symmetric scaling and Dirichlet data.  After it: c64 holds the scaled
// couplings, v64 holds phi~ = D^1/2 g_i on the boundary and 0 inside, and
// cs.dmin the smallest interior diagonal.  red needs NW doubles.
template <int NT>
__device__ void scale2d(CellShared2D &cs, int N, double *c64, double *v64, const double *d64,
                        double *red, int tid) {
  constexpr int NW = NT / 32;
  const int P = N + 3, n = N + 1, lane = tid & 31, warp = tid >> 5;
  // D^-1/2 into v64[.][0] (temporary)
  double dmin_part = 1e300;
  for (int k = tid; k < n * n; k += NT) {
    const int ix = k % n, iy = k / n;
    const int g = (iy + 1) * P + ix + 1;
    const double d = d64[g];
    v64[4 * g] = rsqrt(d);
    if (ix > 0 && iy > 0 && ix < N && iy < N) {
      dmin_part = fmin(dmin_part, d);
      if (!(d > 0.0) || !isfinite(d)) cs.status = MSFEM_CELL_NAN;
    }
  }
  __syncthreads();
  for (int k = tid; k < n * n; k += NT) {
    const int g = (k / n + 1) * P + k % n + 1;
    const double s = v64[4 * g];
    double cc[4];
    ld4(c64, g, cc);
    cc[0] *= s * v64[4 * (g + 1)];
    cc[1] *= s * v64[4 * (g + P + 1)];
    cc[2] *= s * v64[4 * (g + P)];
    cc[3] *= s * v64[4 * (g + P - 1)];
    st4(c64, g, cc);
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) dmin_part = fmin(dmin_part, shfl_xor_d(dmin_part, m));
  if (lane == 0) red[warp] = dmin_part;
  __syncthreads();
  // Dirichlet data phi~_i = D^1/2 g_i (BasisQ1 at the node) in a converged
  // loop over the 4N boundary nodes (FP64 work in a divergent branch costs
  // whole warp instructions); interior 0
  const double invN = 1.0 / (double)N;
  for (int k = tid; k < 4 * N; k += NT) {
    int bx, by;
    boundary_node(k, N, bx, by);
    const int g = (by + 1) * P + bx + 1;
    double x[2], gv[4], t[4];
    bilinear_map(cs.corners, bx == N ? 1.0 : bx * invN, by == N ? 1.0 : by * invN, x);
    q1_eval<2>(cs.q1coef, cs.q1shift, cs.q1iscale, x, gv);
    const double sq = d64[g] * v64[4 * g];
#pragma unroll
    for (int r = 0; r < 4; ++r) t[r] = gv[r] * sq;
    st4(v64, g, t);
  }
  for (int k = tid; k < (N - 1) * (N - 1); k += NT) {
    const double z4[4] = {0.0, 0.0, 0.0, 0.0};
    st4(v64, (k / (N - 1) + 2) * P + k % (N - 1) + 2, z4);
  }
  if (tid == 0) {
    double m = 1e300;
    for (int w = 0; w < NW; ++w) m = fmin(m, red[w]);
    cs.dmin = m;
  }
  __syncthreads();
}

// Dirichlet data and FP32 scaling of the mixed form, which keeps its FP64
// state unscaled: v64 holds phi = g_i on the boundary (BasisQ1 at the node)
// and 0 inside, s32[4 g] the FP32 symmetric scaling d^-1/2 of interior node g
// (0 on the boundary, so scaled couplings to boundary nodes vanish) for the
// FP32 inner solve.  Non-positive or non-finite interior diagonals set
// MSFEM_CELL_NAN.  s32 lives in the FP32 exchange buffer until the inner
// solve overwrites it (every component other than [4 g] stays zero).
template <int NT>
__device__ void prepare2d_unscaled(CellShared2D &cs, int N, double *v64, const double *d64, float *s32,
                                   int tid) {
  const int P = N + 3, n = N + 1;
  // boundary nodes in a loop of their own: FP64 work in divergent branches
  // costs whole warp instructions, so the BasisQ1 evaluation runs converged
  const double invN = 1.0 / (double)N;
  for (int k = tid; k < 4 * N; k += NT) {
    int bx, by;
    boundary_node(k, N, bx, by);
    const int g = (by + 1) * P + bx + 1;
    double x[2], t[4];
    bilinear_map(cs.corners, bx == N ? 1.0 : bx * invN, by == N ? 1.0 : by * invN, x);
    q1_eval<2>(cs.q1coef, cs.q1shift, cs.q1iscale, x, t);
    st4(v64, g, t);
    s32[4 * g] = 0.0f;
  }
  // interior nodes (v64 is already zero there)
  for (int k = tid; k < (N - 1) * (N - 1); k += NT) {
    const int g = (k / (N - 1) + 2) * P + k % (N - 1) + 2;
    const double d = d64[g];
    if (!(d > 0.0) || !isfinite(d)) cs.status = MSFEM_CELL_NAN;
    s32[4 * g] = rsqrtf((float)d);
  }
  __syncthreads();
}

// Interior node k of the ring next to the boundary (k < 4 (N - 2), N >= 3;
// the single interior node for N = 2).
__device__ __forceinline__ void ring_node(int k, int N, int &ix, int &iy) {
  const int m = N - 2;
  if (m <= 0) { ix = 1; iy = 1; }
  else if (k < m) { ix = 1 + k; iy = 1; }
  else if (k < 2 * m) { ix = N - 1; iy = 1 + (k - m); }
  else if (k < 3 * m) { ix = N - 1 - (k - 2 * m); iy = N - 1; }
  else { ix = 1; iy = N - 1 - (k - 3 * m); }
}

// Scaled boundary value phi~ at boundary node (ix, iy).
__device__ __forceinline__ void boundary_value(const CellShared2D &cs, const double *d64, int N,
                                               int P, int ix, int iy, double (&t)[4]) {
  const int g = (iy + 1) * P + ix + 1;
  double x[2], gv[4];
  bilinear_map(cs.corners, ix / (double)N, iy / (double)N, x);
  q1_eval<2>(cs.q1coef, cs.q1shift, cs.q1iscale, x, gv);
  const double d = d64[g];
  const double sq = d * rsqrt(d);
#pragma unroll
  for (int r = 0; r < 4; ++r) t[r] = gv[r] * sq;
}

// Load vector b_k = int f psi_k at node (ix, iy) (diffusion_problem_basis.tpp:
// 219-220): QGauss(2) over the adjacent fine cells.  Constant f on affine
// cells: every fine cell carries f |det| / 4 to each of its vertices.  With f
// tabulated at the Gauss points (p.f_qp), or on general cells, the quadrature
// sum itself, with the per-point |det J| on general cells.
__device__ inline double node_load(const KernelParams &p, const CellShared2D &cs, int N, int ix, int iy) {
  if (cs.affine && !p.f_qp) {
    const double m = (ix == 0 || ix == N ? 1.0 : 2.0) * (iy == 0 || iy == N ? 1.0 : 2.0);
    return p.f_value * 0.25 * cs.absdet * m;
  }
  const double *fq = nullptr;
  const int nfc = N * N;
  if (p.f_qp) fq = p.f_qp + (p.f_qp_offset ? p.f_qp_offset[cs.cell] : (int64_t)cs.cell * 4 * nfc);
  const double invN = 1.0 / (double)N;
  double b = 0.0;
  for (int dy = -1; dy <= 0; ++dy)
    for (int dx = -1; dx <= 0; ++dx) {
      const int cx = ix + dx, cy = iy + dy;
      if (cx < 0 || cy < 0 || cx >= N || cy >= N) continue;
      const int kx = ix - cx, ky = iy - cy;  // local vertex of the node
      const int fc = cy * N + cx;
      double V[8];
      if (!cs.affine) {
        bilinear_map(cs.corners, cx * invN, cy * invN, V + 0);
        bilinear_map(cs.corners, (cx + 1) * invN, cy * invN, V + 2);
        bilinear_map(cs.corners, cx * invN, (cy + 1) * invN, V + 4);
        bilinear_map(cs.corners, (cx + 1) * invN, (cy + 1) * invN, V + 6);
      }
      for (int q = 0; q < 4; ++q) {
        const int qx = q & 1, qy = q >> 1;
        double det = cs.absdet;
        if (!cs.affine) {
          double J00 = 0, J01 = 0, J10 = 0, J11 = 0;
          for (int k = 0; k < 4; ++k) {
            const int vx = k & 1, vy = k >> 1;
            const double gx = (vx ? 1.0 : -1.0) * lval(vy, qy);
            const double gy = (vy ? 1.0 : -1.0) * lval(vx, qx);
            J00 += V[2 * k] * gx; J01 += V[2 * k] * gy;
            J10 += V[2 * k + 1] * gx; J11 += V[2 * k + 1] * gy;
          }
          det = fabs(J00 * J11 - J01 * J10);
        }
        const double f = fq ? fq[q * nfc + fc] : p.f_value;
        b += f * lval(kx, qx) * lval(ky, qy) * 0.25 * det;
      }
    }
  return b;
}

// Epilogue contribution of node (ix, iy) with y = A~ phi~ known there
// (SCALED), or y = A phi with phi unscaled (the mixed form).
template <bool SCALED = true>
__device__ __forceinline__ void epilogue_node(const KernelParams &p, const CellShared2D &cs,
                                              const double *d64, int N, int P, int ix, int iy,
                                              const double (&ph)[4], const double (&y)[4],
                                              double (&acc)[32]) {
  const int g = (iy + 1) * P + ix + 1;
  const double bl = SCALED ? node_load(p, cs, N, ix, iy) * rsqrt(d64[g]) : node_load(p, cs, N, ix, iy);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[4 * i + j] = fma(ph[i], y[j], acc[4 * i + j]);
    acc[16 + i] = fma(ph[i], bl, acc[16 + i]);
  }
}

// Symmetric epilogue of the mixed form: acc[16] holds M_ij for i <= j in the
// order of sym_pair (10 values) and F (4); y = A phi at the node, phi unscaled.
__device__ __forceinline__ void sym_pair(int v, int &i, int &j) {
  // (0,0) (0,1) (0,2) (0,3) (1,1) (1,2) (1,3) (2,2) (2,3) (3,3)
  i = v < 4 ? 0 : v < 7 ? 1 : v < 9 ? 2 : 3;
  j = v < 4 ? v : v < 7 ? v - 3 : v < 9 ? v - 5 : 3;
}
__device__ __forceinline__ void epilogue_node_sym(const KernelParams &p, const CellShared2D &cs, int N,
                                                  int ix, int iy, const double (&ph)[4], const double (&y)[4],
                                                  double (&acc)[16]) {
  const double bl = node_load(p, cs, N, ix, iy);
#pragma unroll
  for (int v = 0; v < 10; ++v) {
    int i, j;
    sym_pair(v, i, j);
    acc[v] = fma(ph[i], y[j], acc[v]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) acc[10 + i] = fma(ph[i], bl, acc[10 + i]);
}

// Final block reduction of the symmetric epilogue (M mirrored) and the output
// writes of the mixed form; the relative residual comes from cs.nu.
template <int NT>
__device__ void epilogue_finish_sym(const KernelParams &p, CellShared2D &cs, int cell, double (&acc)[16],
                                    double *red16, const int (&total_iters)[4], int tid) {
  constexpr int NW = NT / 32;
  const int lane = tid & 31, warp = tid >> 5;
  const double tot = warp_transpose_reduce<16>(acc, lane);
  if ((lane & 1) == 0) red16[warp * 16 + (lane >> 1)] = tot;
  __syncthreads();
  if (warp == 0) {
    double s = 0.0;
    if (lane < 16)
      for (int w = 0; w < NW; ++w) s += red16[w * 16 + lane];
    if (lane < 10) {
      int i, j;
      sym_pair(lane, i, j);
      p.M[(int64_t)cell * 16 + 4 * i + j] = s;
      p.M[(int64_t)cell * 16 + 4 * j + i] = s;
    } else if (lane < 14) {
      p.F[(int64_t)cell * 4 + (lane - 10)] = s;
    }
    double rel = 0.0;
    if (lane < 4) {
      const double bb = cs.bb[lane];
      const double nu = cs.nu[lane];
      rel = bb > 0.0 ? sqrt(nu / bb) : sqrt(nu);
    }
#pragma unroll
    for (int m = 2; m >= 1; m >>= 1) rel = fmax(rel, shfl_xor_d(rel, m));
    if (lane < 4 && p.iters) p.iters[(int64_t)cell * 4 + lane] = total_iters[lane];
    if (lane == 0) {
      int st = cs.status;
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

// Final block reduction of the 32 epilogue values and the output writes.
// acc: M (16), F (4), interior ||A phi||^2 (4) unless use_nu, then cs.nu.
template <int NT, bool MIXED>
__device__ void epilogue_finish(const KernelParams &p, CellShared2D &cs, int cell, double (&acc)[32],
                                double *red32v, bool use_nu, const int (&total_iters)[4], int tid) {
  constexpr int NW = NT / 32;
  const int lane = tid & 31, warp = tid >> 5;
  const double tot = warp_transpose_reduce<32>(acc, lane);
  red32v[warp * 32 + lane] = tot;
  __syncthreads();
  if (warp == 0) {
    double s = 0.0;
    for (int w = 0; w < NW; ++w) s += red32v[w * 32 + lane];
    if (lane < 16) p.M[(int64_t)cell * 16 + lane] = s;
    else if (lane < 20) p.F[(int64_t)cell * 4 + (lane - 16)] = s;
    double rel = 0.0;
    if (lane >= 20 && lane < 24) {
      const double bb = cs.bb[lane - 20];
      const double nu = use_nu ? cs.nu[lane - 20] : s;
      rel = bb > 0.0 ? sqrt(nu / bb) : sqrt(nu);
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) rel = fmax(rel, shfl_xor_d(rel, m));
    if (lane < 4 && p.iters) {
      const int itv = cs.iters[lane];
      int out;
      if (MIXED) out = total_iters[lane];
      else out = itv >= 0 ? itv : (itv <= -1000000 ? -itv - 1000000 : -itv);
      p.iters[(int64_t)cell * 4 + lane] = out;
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

// Basis output phi = D^-1/2 phi~ (lexicographic nodes), when requested;
// SCALED = false: v64 holds phi itself.
template <int NT, bool SCALED = true>
__device__ void write_basis(const KernelParams &p, int cell, int N, const double *v64,
                            const double *d64, int tid) {
  if (!p.basis) return;
  const int P = N + 3, n = N + 1;
  double *out = p.basis + (p.basis_offset ? p.basis_offset[cell] : (int64_t)cell * 4 * n * n);
  for (int k = tid; k < n * n; k += NT) {
    const int g = (k / n + 1) * P + k % n + 1;
    double ph[4];
    ld4(v64, g, ph);
    const double s = SCALED ? rsqrt(d64[g]) : 1.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) out[(int64_t)i * n * n + k] = ph[i] * s;
  }
}

// ===========================================================================
// Plain FP64 form
// ===========================================================================
template <int NMAX, int NT>
__global__ void __launch_bounds__(NT, 2)
msfem2d_kernel(const KernelParams p) {
  using L = Smem2D<NMAX>;
  constexpr int NW = NT / 32;
  constexpr int NPT = ((NMAX - 1) * (NMAX - 1) + NT - 1) / NT;  // interior nodes per thread
  static_assert(4 * (NMAX - 2) <= NT, "the boundary-adjacent ring takes one node per thread");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *c64 = reinterpret_cast<double *>(smem_raw + L::kC64);
  double *v64 = reinterpret_cast<double *>(smem_raw + L::kV64);
  double *d64 = reinterpret_cast<double *>(smem_raw + L::kD64);
  __shared__ CellShared2D cs;
  __shared__ double red[2][NW * 8];
  __shared__ double redE[NW * 32];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int zero_iters[4] = {0, 0, 0, 0};

  for (;;) {
    if (tid == 0) {
      const unsigned wi = atomicAdd(p.queue, 1u);
      cs.cell = wi < (unsigned)p.n_cells ? (p.order ? p.order[wi] : (int)wi) : -1;
    }
    __syncthreads();
    const int cell = cs.cell;
    if (cell < 0) break;
    const int N = p.n_fine ? p.n_fine[cell] : p.n_fine_uniform;
    const int P = N + 3, n = N + 1, nI = (N - 1) * (N - 1);

    if (cell_begin<NMAX, NT>(p, cs, cell, N, c64, v64, d64, nullptr, tid) != MSFEM_CELL_CONVERGED) {
      cell_report_bad(p, cs, cell, tid);
      __syncthreads();
      continue;
    }
    assemble2d<NT>(p, cs, cell, N, c64, d64, tid);
    if (cs.status != MSFEM_CELL_CONVERGED) {
      cell_report_bad(p, cs, cell, tid);
      __syncthreads();
      continue;
    }
    scale2d<NT>(cs, N, c64, v64, d64, red[0], tid);

    // ---------------- right-hand sides ------------------------------------
    int gidx[NPT];
    double dloc[NPT];
#pragma unroll
    for (int j = 0; j < NPT; ++j) {
      const int k = tid + j * NT;
      gidx[j] = k < nI ? (1 + k / (N - 1) + 1) * P + (1 + k % (N - 1)) + 1 : -1;
      dloc[j] = gidx[j] >= 0 ? d64[gidx[j]] : 0.0;
    }
    // b~ = -(A~ phi~)_I vanishes away from the boundary (phi~ is zero
    // inside): one converged pass over the 4 (N - 2) boundary-adjacent nodes
    // computes it, and the node owners pick it up from v64's (zero) interior
    double rr[NPT][4];   // FP64 residual (scaled)
    double bbp[4] = {0.0, 0.0, 0.0, 0.0};
    {
      const int nring = N >= 3 ? 4 * (N - 2) : (N == 2 ? 1 : 0);
      double bk[4] = {0.0, 0.0, 0.0, 0.0};
      int gk = -1;
      if (tid < nring) {
        int rx, ry;
        ring_node(tid, N, rx, ry);
        gk = (ry + 1) * P + rx + 1;
        stencil9<double>(c64, v64, gk, P, bk);
        const double dk = d64[gk];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          bk[r] = -bk[r];
          bbp[r] = (bk[r] * dk) * bk[r];
        }
      }
      warp_partials<4>(bbp, red[1], warp, lane);
      __syncthreads();  // every stencil read of v64 is done
      if (gk >= 0) st4(v64, gk, bk);
      __syncthreads();
#pragma unroll
      for (int j = 0; j < NPT; ++j) {
#pragma unroll
        for (int r = 0; r < 4; ++r) rr[j][r] = 0.0;
        if (gidx[j] >= 0) ld4(v64, gidx[j], rr[j]);
      }
    }
    if (warp == 0) {
      const double t = warp_finish<4>(red[1], NW, lane);
      if (lane < 4) {
        cs.bb[lane] = t;
        cs.bthr[lane] = p.tol_abs ? 1.0 : t;
      }
    }
    // warm start: x~0 = D^1/2 phi_warm on the interior, r0 = -(A~ phi~0)_I
    const bool warm = p.warm_basis != nullptr;
    double xr[NPT][4], qr[NPT][4];
#pragma unroll
    for (int j = 0; j < NPT; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) { xr[j][r] = 0.0; qr[j][r] = 0.0; }
    if (warm) {
      const double *wb = p.warm_basis + (p.basis_offset ? p.basis_offset[cell] : (int64_t)cell * 4 * n * n);
      __syncthreads();
#pragma unroll
      for (int j = 0; j < NPT; ++j)
        if (gidx[j] >= 0) {
          const int g = gidx[j];
          const int node = (g / P - 1) * n + (g % P - 1);
          const double sq = sqrt(dloc[j]);
#pragma unroll
          for (int r = 0; r < 4; ++r) xr[j][r] = __ldg(wb + (int64_t)r * n * n + node) * sq;
          st4(v64, g, xr[j]);
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
    // v64 becomes p~ (zero on the boundary ring)
    for (int k = tid; k < 4 * N; k += NT) {
      int ix, iy;
      boundary_node(k, N, ix, iy);
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
      const double t = warp_finish<8>(red[0], NW, lane);
      const double nu = shfl_xor_d(t, 4);  // lane r (<4) gets value 4+r
      if (lane < 4) {
        cs.rho[lane] = t;
        const bool conv = nu <= tol2 * cs.bthr[lane];
        cs.active[lane] = !conv;
        cs.iters[lane] = 0;
        cs.beta[lane] = 0.0;
      }
      __syncwarp();
      if (lane == 0) {
        int any = 0, nn2 = 0;
        for (int r = 0; r < 4; ++r) {
          any |= cs.active[r];
          if (cs.active[r] && cs.dmin * cs.rho[r] <= 100.0 * tol2 * cs.bthr[r]) nn2 = 1;
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
        const double t = warp_finish<4>(red[1], NW, lane);
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
      const double al[4] = {cs.alpha[0], cs.alpha[1], cs.alpha[2], cs.alpha[3]};
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
          t = warp_finish<8>(red[0], NW, lane);
          nu = shfl_xor_d(t, 4);
        } else {
          t = warp_finish<4>(red[0], NW, lane);
        }
        if (lane < 4) {
          double b = 0.0;
          if (cs.active[lane]) {
            if (!isfinite(t)) {
              cs.active[lane] = 0;
              cs.iters[lane] = -it;
            } else if (t == 0.0 || (need_nu && nu <= tol2 * cs.bthr[lane])) {
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
            if (cs.active[r] && cs.dmin * cs.rho[r] <= 100.0 * tol2 * cs.bthr[r]) nn2 = 1;
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
      boundary_node(k, N, ix, iy);
      double t[4];
      boundary_value(cs, d64, N, P, ix, iy, t);
      st4(v64, (iy + 1) * P + ix + 1, t);
    }
    __syncthreads();

    // ---------------- epilogue: M, F, true residual ----------------------
    double acc[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) acc[i] = 0.0;
    for (int k = tid; k < n * n; k += NT) {
      const int ix = k % n, iy = k / n;
      const int g = (iy + 1) * P + ix + 1;
      double y[4], ph[4];
      stencil9<double>(c64, v64, g, P, y);
      ld4(v64, g, ph);
      epilogue_node(p, cs, d64, N, P, ix, iy, ph, y, acc);
      if (ix > 0 && iy > 0 && ix < N && iy < N) {
        const double d = d64[g];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[20 + j] = fma(y[j] * d, y[j], acc[20 + j]);
      }
    }
    write_basis<NT>(p, cell, N, v64, d64, tid);
    epilogue_finish<NT, false>(p, cs, cell, acc, redE, false, zero_iters, tid);
  }
}


// ---------------------------------------------------------------------------
// Strip helpers of the mixed form (thread = S consecutive rows of one column)
// ---------------------------------------------------------------------------
// FP32 couplings of a strip row: E, W, N, S, NE, SW, NW, SE.
template <int S>
struct StripCoup {
  float cE[S], cW[S], cN[S], cS[S], cNE[S], cSW[S], cNW[S], cSE[S];
};

// y = A~ x on the strip's own rows: own-column neighbours from the registers
// x, the two neighbour columns and the two halo rows from buf ([G][4] FP32,
// zero outside the interior).  Each value of a neighbour column is loaded
// once and scattered into the (up to three) rows that couple to it.
template <int S>
__device__ __forceinline__ void strip_apply(const float *__restrict__ buf, int g0, int P, int ns,
                                            const StripCoup<S> &c, const float (&x)[S][4], float (&y)[S][4]) {
#pragma unroll
  for (int s = 0; s < S; ++s)
#pragma unroll
    for (int r = 0; r < 4; ++r) y[s][r] = x[s][r];
  if (ns <= 0) return;
  float t4[4];
  ld4(buf, g0 - P, t4);  // row below the strip
#pragma unroll
  for (int r = 0; r < 4; ++r) y[0][r] = fmaf(c.cS[0], t4[r], y[0][r]);
#pragma unroll
  for (int s = 0; s < S; ++s) {
    if (s < ns) {
      if (s > 0) {
#pragma unroll
        for (int r = 0; r < 4; ++r) y[s][r] = fmaf(c.cS[s], x[s - 1][r], y[s][r]);
      }
      if (s + 1 < ns) {
#pragma unroll
        for (int r = 0; r < 4; ++r) y[s][r] = fmaf(c.cN[s], x[s + 1][r], y[s][r]);
      } else {
        ld4(buf, g0 + (s + 1) * P, t4);  // row above the strip
#pragma unroll
        for (int r = 0; r < 4; ++r) y[s][r] = fmaf(c.cN[s], t4[r], y[s][r]);
      }
    }
  }
#pragma unroll
  for (int t = -1; t <= S; ++t) {
    if (t <= ns) {
      ld4(buf, g0 + t * P - 1, t4);  // left column, row s0 + t
      if (t >= 1 && t - 1 < ns) {
#pragma unroll
        for (int r = 0; r < 4; ++r) y[t - 1][r] = fmaf(c.cNW[t - 1], t4[r], y[t - 1][r]);
      }
      if (t >= 0 && t < ns) {
#pragma unroll
        for (int r = 0; r < 4; ++r) y[t][r] = fmaf(c.cW[t], t4[r], y[t][r]);
      }
      if (t + 1 < ns && t + 1 < S) {
#pragma unroll
        for (int r = 0; r < 4; ++r) y[t + 1][r] = fmaf(c.cSW[t + 1], t4[r], y[t + 1][r]);
      }
      ld4(buf, g0 + t * P + 1, t4);  // right column, row s0 + t
      if (t >= 1 && t - 1 < ns) {
#pragma unroll
        for (int r = 0; r < 4; ++r) y[t - 1][r] = fmaf(c.cNE[t - 1], t4[r], y[t - 1][r]);
      }
      if (t >= 0 && t < ns) {
#pragma unroll
        for (int r = 0; r < 4; ++r) y[t][r] = fmaf(c.cE[t], t4[r], y[t][r]);
      }
      if (t + 1 < ns && t + 1 < S) {
#pragma unroll
        for (int r = 0; r < 4; ++r) y[t + 1][r] = fmaf(c.cSE[t + 1], t4[r], y[t + 1][r]);
      }
    }
  }
}

// y[0..1] += c x[0..1] and y[2..3] += c x[2..3] as two packed FP32 pair
// FMAs (FFMA2): the four right-hand sides of a node in two instructions.
// (Measured on the polynomial steps' stencil: 3 % faster with degree 5;
// the same packing of the CG vector updates made the loop slower.)
__device__ __forceinline__ void fma4_x2(float c, const float (&x)[4], float (&y)[4]) {
  const float2 cc = make_float2(c, c);
  const float2 a = __ffma2_rn(cc, make_float2(x[0], x[1]), make_float2(y[0], y[1]));
  const float2 b = __ffma2_rn(cc, make_float2(x[2], x[3]), make_float2(y[2], y[3]));
  y[0] = a.x; y[1] = a.y; y[2] = b.x; y[3] = b.y;
}

// strip_apply with packed pair FMAs (same operations, same rounding).
template <int S>
__device__ __forceinline__ void strip_apply_x2(const float *__restrict__ buf, int g0, int P, int ns,
                                               const StripCoup<S> &c, const float (&x)[S][4], float (&y)[S][4]) {
#pragma unroll
  for (int s = 0; s < S; ++s)
#pragma unroll
    for (int r = 0; r < 4; ++r) y[s][r] = x[s][r];
  if (ns <= 0) return;
  float t4[4];
  ld4(buf, g0 - P, t4);  // row below the strip
  fma4_x2(c.cS[0], t4, y[0]);
#pragma unroll
  for (int s = 0; s < S; ++s) {
    if (s < ns) {
      if (s > 0) fma4_x2(c.cS[s], x[s - 1], y[s]);
      if (s + 1 < ns) {
        fma4_x2(c.cN[s], x[s + 1], y[s]);
      } else {
        ld4(buf, g0 + (s + 1) * P, t4);  // row above the strip
        fma4_x2(c.cN[s], t4, y[s]);
      }
    }
  }
#pragma unroll
  for (int u = -1; u <= S; ++u) {
    if (u <= ns) {
      ld4(buf, g0 + u * P - 1, t4);  // left column, row s0 + u
      if (u >= 1 && u - 1 < ns) fma4_x2(c.cNW[u - 1], t4, y[u - 1]);
      if (u >= 0 && u < ns) fma4_x2(c.cW[u], t4, y[u]);
      if (u + 1 < ns && u + 1 < S) fma4_x2(c.cSW[u + 1], t4, y[u + 1]);
      ld4(buf, g0 + u * P + 1, t4);  // right column, row s0 + u
      if (u >= 1 && u - 1 < ns) fma4_x2(c.cNE[u - 1], t4, y[u - 1]);
      if (u >= 0 && u < ns) fma4_x2(c.cE[u], t4, y[u]);
      if (u + 1 < ns && u + 1 < S) fma4_x2(c.cSE[u + 1], t4, y[u + 1]);
    }
  }
}

template <int S>
__device__ __forceinline__ void strip_store(float *__restrict__ buf, int g0, int P, int ns, const float (&x)[S][4]) {
#pragma unroll
  for (int s = 0; s < S; ++s)
    if (s < ns) st4(buf, g0 + s * P, x[s]);
}

// Block sum of K FP32 values; every thread ends with the K totals.  red
// holds NW * K floats; callers alternate two such arrays so that a sum can
// follow the previous one without an extra barrier.
template <int K, int NW>
__device__ __forceinline__ void block_sum_f(float (&v)[K], float *red, int warp, int lane) {
  const float t = warp_transpose_reduce<K>(v, lane);
  constexpr int SPAN = 32 / K;
  if ((lane & (SPAN - 1)) == 0) red[warp * K + lane / SPAN] = t;
  __syncthreads();
  float s = 0.f;
  for (int i = lane; i < NW * K; i += 32) s += red[i];
  // lane l now holds partial sums of value l % K
#pragma unroll
  for (int m = K; m < 32; m <<= 1) s += shfl_xor_d(s, m);
#pragma unroll
  for (int j = 0; j < K; ++j) v[j] = __shfl_sync(0xffffffffu, s, j);
}

// ===========================================================================
// Mixed form: FP64 residual refinement around an FP32 CG.  Thread t owns
// interior column ix = 1 + t % (N-1) and rows s0 .. s0+S-1 of it,
// s0 = 1 + S (t / (N-1)): the strip's own search-direction values stay in
// registers, only its two neighbour columns and two halo rows come from
// shared memory.
//
// Inner preconditioner: M = 0 Jacobi scaling only; M > 0 a Chebyshev
// polynomial of degree M - 1 on the scaled operator; CH > 0 (with M > 0) a
// symmetric two-level V-cycle: Chebyshev smoothing of degree M - 1 before and
// after a Galerkin coarse-grid correction on the bilinear coarse space of
// spacing CH fine cells (used where CH divides N and the coarse grid has
// interior nodes; other cells take the smoother alone).
// ===========================================================================
template <int NMAX, int NT, int S, int MINB, int M, int CH = 0>
__global__ void __launch_bounds__(NT, MINB)
msfem2d_mixed_kernel(const KernelParams p) {
  using L = Smem2D<NMAX>;
  using C = Coarse2D<NMAX, CH>;
  constexpr int NW = NT / 32;
  // threads per row-block of strips: the interior columns rounded up to a
  // multiple of 8 lanes (one quarter-warp of 16-byte accesses)
  constexpr int kSlots = (NMAX - 1 + 7) / 8 * 8;
  static_assert(kSlots * ((NMAX - 1 + S - 1) / S) <= NT, "strips must cover the interior");
  // the coarse grid's rows are the strips' row-blocks and its columns fall
  // within one warp of strips; two exchange buffers
  static_assert(CH == 0 || (CH == S && kSlots == 32 && MINB == 1 && M >= 2), "two-level shape");
  static_assert(CH == 0 || 4 * C::NI <= NT, "four threads per coarse node in the coarse solve");
  static_assert(NW * 32 * sizeof(double) <= 16 * L::G, "epilogue partials fit in v32");
  static_assert(4 * (NMAX - 2) <= NT, "the boundary-adjacent ring takes one node per thread");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *c64 = reinterpret_cast<double *>(smem_raw + L::kC64);
  double *v64 = reinterpret_cast<double *>(smem_raw + L::kV64);
  double *d64 = reinterpret_cast<double *>(smem_raw + L::kD64);
  float *v32 = reinterpret_cast<float *>(smem_raw + L::kV32);
  float *v32b = reinterpret_cast<float *>(smem_raw + L::kV32B);  // used only when M > 0
  __shared__ CellShared2D cs;
  __shared__ double red[2][NW * 8];
  __shared__ float red32[2][NW * 8];
  __shared__ float gersh_part[NW];

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
    const int P = N + 3, n = N + 1;

    if (cell_begin<NMAX, NT>(p, cs, cell, N, c64, v64, d64, v32, tid) != MSFEM_CELL_CONVERGED) {
      cell_report_bad(p, cs, cell, tid);
      __syncthreads();
      continue;
    }
    if constexpr (M > 0 && MINB < 2)
      for (int i = tid; i < 4 * (N + 3) * (N + 3); i += NT) v32b[i] = 0.0f;
    assemble2d<NT, true>(p, cs, cell, N, c64, d64, tid);
    if (cs.status != MSFEM_CELL_CONVERGED) {
      cell_report_bad(p, cs, cell, tid);
      __syncthreads();
      continue;
    }
    // The FP64 state stays unscaled (operator with its diagonal, phi = g on
    // the boundary); only the FP32 inner solve works on the symmetrically
    // scaled operator, with the scaling d^-1/2 computed in FP32.
    prepare2d_unscaled<NT>(cs, N, v64, d64, v32, tid);

    // strip of this thread: SLOTS threads per row-block of strips (lane =
    // column), so a quarter-warp never straddles two row-blocks and every
    // 16-byte shared access of the strip loops is one contiguous wavefront
    const int ncol = N - 1;
    const int nstrip = ncol > 0 ? (ncol + S - 1) / S : 0;
    const int col = tid % kSlots, blk = tid / kSlots;
    const bool own = col < ncol && blk < nstrip;
    const int ix = own ? 1 + col : 1;
    const int s0 = own ? 1 + S * blk : 1;
    const int ns = own ? min(S, N - s0) : 0;
    const int g0 = (s0 + 1) * P + ix + 1;

    // FP64 right-hand sides b = -(A phi)_I (and warm start).  phi is zero
    // inside, so b vanishes at every node not next to the boundary: one
    // converged pass over that ring of 4 (N - 2) nodes computes it (one node
    // per thread), and the strip owners pick it up from the interior entries
    // of v64, which are zero until then.
    double r64[S][4];
    double bbp[4] = {0.0, 0.0, 0.0, 0.0};
    const int nring = N >= 3 ? 4 * (N - 2) : (N == 2 ? 1 : 0);
    double bk[4] = {0.0, 0.0, 0.0, 0.0};
    int gk = -1;
    if (tid < nring) {
      int rx, ry;
      ring_node(tid, N, rx, ry);
      gk = (ry + 1) * P + rx + 1;
      stencil9<double>(c64, v64, gk, P, bk);  // own value 0: no diagonal term
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        bk[r] = -bk[r];
        bbp[r] = bk[r] * bk[r];
      }
    }
    warp_partials<4>(bbp, red[1], warp, lane);
    __syncthreads();  // every stencil read of v64 is done
    if (gk >= 0) st4(v64, gk, bk);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < S; ++s) {
#pragma unroll
      for (int r = 0; r < 4; ++r) r64[s][r] = 0.0;
      if (s < ns) {
        ld4(v64, g0 + s * P, r64[s]);
        const double z4[4] = {0.0, 0.0, 0.0, 0.0};
        st4(v64, g0 + s * P, z4);  // the iterate starts at zero
      }
    }
    if (warp == 0) {
      const double t = warp_finish<4>(red[1], NW, lane);
      if (lane < 4) {
        cs.bb[lane] = t;
        cs.bthr[lane] = p.tol_abs ? 1.0 : t;
      }
    }
    if (p.warm_basis != nullptr) {
      const double *wb = p.warm_basis + (p.basis_offset ? p.basis_offset[cell] : (int64_t)cell * 4 * n * n);
      __syncthreads();
#pragma unroll
      for (int s = 0; s < S; ++s)
        if (s < ns) {
          const int g = g0 + s * P;
          const int node = (s0 + s) * n + ix;
          double t[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) t[r] = __ldg(wb + (int64_t)r * n * n + node);
          st4(v64, g, t);
        }
      __syncthreads();
#pragma unroll
      for (int s = 0; s < S; ++s)
        if (s < ns) {
          double y[4];
          stencil9_unscaled(c64, d64, v64, g0 + s * P, P, y);
#pragma unroll
          for (int r = 0; r < 4; ++r) r64[s][r] = -y[r];
        }
    }
    // FP32 couplings of the strip, symmetrically scaled in FP32 (s = d^-1/2
    // from v32[4 g], 0 on the boundary): E, W, N, S, NE, SW, NW, SE of every
    // row; sown the strip's own scaling for the residual and the correction
    StripCoup<S> cp;
    float sown[S];
    float gmax = 0.0f;  // Gershgorin bound of A~ (unit diagonal) over the strip
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const int g = g0 + s * P;
      const bool v = s < ns;
      const float sg = v ? v32[4 * g] : 0.f;
      sown[s] = sg;
      cp.cE[s] = v ? (float)(c64[4 * g + 0]) * sg * v32[4 * (g + 1)] : 0.f;
      cp.cNE[s] = v ? (float)(c64[4 * g + 1]) * sg * v32[4 * (g + P + 1)] : 0.f;
      cp.cN[s] = v ? (float)(c64[4 * g + 2]) * sg * v32[4 * (g + P)] : 0.f;
      cp.cNW[s] = v ? (float)(c64[4 * g + 3]) * sg * v32[4 * (g + P - 1)] : 0.f;
      cp.cW[s] = v ? (float)(c64[4 * (g - 1) + 0]) * sg * v32[4 * (g - 1)] : 0.f;
      cp.cS[s] = v ? (float)(c64[4 * (g - P) + 2]) * sg * v32[4 * (g - P)] : 0.f;
      cp.cSW[s] = v ? (float)(c64[4 * (g - P - 1) + 1]) * sg * v32[4 * (g - P - 1)] : 0.f;
      cp.cSE[s] = v ? (float)(c64[4 * (g - P + 1) + 3]) * sg * v32[4 * (g - P + 1)] : 0.f;
      gmax = fmaxf(gmax, 1.0f + fabsf(cp.cE[s]) + fabsf(cp.cW[s]) + fabsf(cp.cN[s]) + fabsf(cp.cS[s]) +
                             fabsf(cp.cNE[s]) + fabsf(cp.cSW[s]) + fabsf(cp.cNW[s]) + fabsf(cp.cSE[s]));
    }
    // Chebyshev interval [b / ratio, b] of the polynomial preconditioner: b
    // the Gershgorin bound (>= lambda_max, so the polynomial stays positive
    // on the spectrum and the preconditioner SPD)
    float cheb_c1[M > 0 ? M : 1], cheb_c2[M > 0 ? M : 1], cheb_inv_theta = 1.0f;
    if constexpr (M > 0) {
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) gmax = fmaxf(gmax, __shfl_xor_sync(0xffffffffu, gmax, m));
      if (lane == 0) gersh_part[warp] = gmax;
      __syncthreads();
      float bmax = 1.0f;
      for (int w = 0; w < NW; ++w) bmax = fmaxf(bmax, gersh_part[w]);
      const float amin = bmax / fmaxf(p.cheb_ratio, 1.5f);
      const float theta = 0.5f * (bmax + amin), delta = 0.5f * (bmax - amin), sigma = theta / delta;
      cheb_inv_theta = 1.0f / theta;
      float rho_prev = 1.0f / sigma;
      cheb_c1[0] = cheb_c2[0] = 0.0f;
#pragma unroll
      for (int k = 1; k < M; ++k) {
        const float rho_k = 1.0f / (2.0f * sigma - rho_prev);
        cheb_c1[k] = rho_k * rho_prev;
        cheb_c2[k] = 2.0f * rho_k / delta;
        rho_prev = rho_k;
      }
    }

    // ---- two-level preconditioner (CH > 0): coarse grid of ncg intervals of
    // CH fine cells; coarse row j at fine row CH j is the boundary between
    // strip row-blocks j - 1 and j, so each strip sees exactly coarse rows
    // blk and blk + 1, with bilinear weights (CH - 1 - s) / CH and (s + 1) / CH
    constexpr int kCH = CH > 0 ? CH : 1;  // CH as a divisor (the CH = 0 shapes compile this code unused)
    const int ncg = (CH > 0 && N % kCH == 0) ? N / kCH : 0;
    const bool coarse = CH > 0 && ncg >= 2;
    const int nI = coarse ? (ncg - 1) * (ncg - 1) : 0;
    float4 *ub = reinterpret_cast<float4 *>(smem_raw + C::kUB);
    float4 *rcs = reinterpret_cast<float4 *>(smem_raw + C::kRC);
    float4 *ecz = reinterpret_cast<float4 *>(smem_raw + C::kEC);
    const float *Aci = reinterpret_cast<const float *>(smem_raw + C::kA0);
    // D^1/2 of the strip (the coarse space in scaled variables is D^1/2 P)
    float sq[S];
#pragma unroll
    for (int s = 0; s < S; ++s) sq[s] = sown[s] > 0.0f ? 1.0f / sown[s] : 0.0f;
    // bilinear x weights of the strip's column: coarse columns cxl, cxl + 1
    const int cxl = CH > 0 ? ix / kCH : 0;
    const float wxh = CH > 0 ? (float)(ix - CH * cxl) * (1.0f / kCH) : 0.0f, wxl = 1.0f - wxh;
    // one stencil pass y = A~ x through the exchange buffers v32 / v32b in
    // turn: one barrier per pass, since a buffer is written again only after
    // the barrier that follows every read of it
    int bsel = 0;
    auto pass = [&](const float (&x)[S][4], float (&y)[S][4]) {
      float *bk = bsel ? v32b : v32;
      bsel ^= 1;
      strip_store<S>(bk, g0, P, ns, x);
      __syncthreads();
      strip_apply_x2<S>(bk, g0, P, ns, cp, x, y);
    };
    // rcs = (D^1/2 P)^T e: each strip folds its rows onto its two coarse
    // rows, then one thread per coarse node sums the 2 CH - 1 columns of
    // the two row-blocks next to it (measured faster than a shuffle window
    // sum inside each row-block, whose partials the coarse solve would
    // then have to combine)
    auto restrict_c = [&](const float (&e)[S][4], bool closing_barrier = true) {
      if (own) {
        float lo[4] = {0.f, 0.f, 0.f, 0.f}, hi[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int s = 0; s < S; ++s) {
          const float wl = (float)(CH - 1 - s) * (1.0f / kCH) * sq[s];
          const float wh = (float)(s + 1) * (1.0f / kCH) * sq[s];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            lo[r] = fmaf(wl, e[s][r], lo[r]);
            hi[r] = fmaf(wh, e[s][r], hi[r]);
          }
        }
        ub[blk * 33 + col] = make_float4(lo[0], lo[1], lo[2], lo[3]);
        ub[(C::NC + blk) * 33 + col] = make_float4(hi[0], hi[1], hi[2], hi[3]);
      }
      __syncthreads();
      if (tid < nI) {
        const int cy = 1 + tid / (ncg - 1), cx = 1 + tid % (ncg - 1);
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int d = 1 - CH; d <= CH - 1; ++d) {
          const float w = (float)(CH - (d < 0 ? -d : d)) * (1.0f / kCH);
          const int c = CH * cx + d - 1;  // lane of fine column CH cx + d
          const float4 u0 = ub[cy * 33 + c], u1 = ub[(C::NC + cy - 1) * 33 + c];
          a.x = fmaf(w, u0.x + u1.x, a.x);
          a.y = fmaf(w, u0.y + u1.y, a.y);
          a.z = fmaf(w, u0.z + u1.z, a.z);
          a.w = fmaf(w, u0.w + u1.w, a.w);
        }
        rcs[tid] = a;
      }
      if (closing_barrier) __syncthreads();  // uniform argument
    };
    // cr = D^1/2 P Ac^-1 rcs: four threads per coarse node (a quarter of the
    // dense row each), then bilinear prolongation from the strip's corners
    auto coarse_solve = [&](float (&cr)[S][4]) {
      if (tid < ((4 * nI + 31) & ~31)) {  // whole warps (shuffles below)
        const int i = tid >> 2, q = tid & 3;
        float a[4] = {0.f, 0.f, 0.f, 0.f};
        if (i < nI)
#pragma unroll 4
          for (int j = q; j < nI; j += 4) {
            const float w = Aci[i * nI + j];
            const float4 v = rcs[j];
            a[0] = fmaf(w, v.x, a[0]);
            a[1] = fmaf(w, v.y, a[1]);
            a[2] = fmaf(w, v.z, a[2]);
            a[3] = fmaf(w, v.w, a[3]);
          }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          a[r] += __shfl_xor_sync(0xffffffffu, a[r], 1);
          a[r] += __shfl_xor_sync(0xffffffffu, a[r], 2);
        }
        if (q == 0 && i < nI)
          ecz[(1 + i / (ncg - 1)) * (ncg + 1) + 1 + i % (ncg - 1)] = make_float4(a[0], a[1], a[2], a[3]);
      }
      __syncthreads();
      float bo[4] = {0.f, 0.f, 0.f, 0.f}, to[4] = {0.f, 0.f, 0.f, 0.f};
      if (own) {
        const float4 e00 = ecz[blk * (ncg + 1) + cxl], e01 = ecz[blk * (ncg + 1) + cxl + 1];
        const float4 e10 = ecz[(blk + 1) * (ncg + 1) + cxl], e11 = ecz[(blk + 1) * (ncg + 1) + cxl + 1];
        bo[0] = wxl * e00.x + wxh * e01.x; bo[1] = wxl * e00.y + wxh * e01.y;
        bo[2] = wxl * e00.z + wxh * e01.z; bo[3] = wxl * e00.w + wxh * e01.w;
        to[0] = wxl * e10.x + wxh * e11.x; to[1] = wxl * e10.y + wxh * e11.y;
        to[2] = wxl * e10.z + wxh * e11.z; to[3] = wxl * e10.w + wxh * e11.w;
      }
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const float wh = (float)(s + 1) * (1.0f / kCH), wl = 1.0f - wh;
#pragma unroll
        for (int r = 0; r < 4; ++r) cr[s][r] = sq[s] * fmaf(wl, bo[r], wh * to[r]);
      }
    };
    if constexpr (CH > 0) {
      if (coarse) {  // uniform over the CTA
        float *a0 = reinterpret_cast<float *>(smem_raw + C::kA0);
        float *a1 = reinterpret_cast<float *>(smem_raw + C::kA1);
        for (int i = tid; i < nI * nI; i += NT) a1[i] = 0.0f;
        for (int i = tid; i < (ncg + 1) * (ncg + 1); i += NT) ecz[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        // Galerkin Ac = (D^1/2 P)^T A~ (D^1/2 P) by probing: coarse node J
        // has colour (jx mod 3) + 3 (jy mod 3), and one stencil pass over the
        // sum of the coarse functions of 4 colours (one per RHS lane) gives,
        // restricted to node I, the entry of the colour's one J next to I
#pragma unroll 1
        for (int pp = 0; pp < 3; ++pp) {
          float v[S][4];
#pragma unroll
          for (int s = 0; s < S; ++s)
#pragma unroll
            for (int r = 0; r < 4; ++r) v[s][r] = 0.0f;
          if (own) {
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
              for (int a = 0; a < 2; ++a) {
                const int jx = cxl + a, jy = blk + b;
                if (jx < 1 || jx > ncg - 1 || jy < 1 || jy > ncg - 1) continue;
                const int colour = jx % 3 + 3 * (jy % 3) - 4 * pp;
                const float wx = a ? wxh : wxl;
#pragma unroll
                for (int s = 0; s < S; ++s) {
                  const float wy = (float)(b ? s + 1 : CH - 1 - s) * (1.0f / kCH);
#pragma unroll
                  for (int r = 0; r < 4; ++r)
                    if (colour == r) v[s][r] = fmaf(sq[s] * wx, wy, v[s][r]);
                }
              }
          }
          float y[S][4];
          pass(v, y);
          restrict_c(y, false);  // rcs[tid] is read back by the thread that wrote it
          if (tid < nI) {
            const int Ix = 1 + tid % (ncg - 1), Iy = 1 + tid / (ncg - 1);
            const float4 rr = rcs[tid];
            const float rv4[4] = {rr.x, rr.y, rr.z, rr.w};
#pragma unroll
            for (int r = 0; r < 4; ++r) {
              const int c = 4 * pp + r;
              if (c >= 9) continue;
              const int jx = Ix - 1 + ((c % 3 - (Ix - 1) % 3 + 3) % 3);
              const int jy = Iy - 1 + ((c / 3 - (Iy - 1) % 3 + 3) % 3);
              if (jx >= 1 && jx <= ncg - 1 && jy >= 1 && jy <= ncg - 1)
                a1[tid * nI + (jy - 1) * (ncg - 1) + jx - 1] = rv4[r];
            }
          }
        }
        __syncthreads();
        // Ac^-1 without block barriers per pivot.  In the lexicographic
        // coarse numbering Ac is banded (bandwidth ncg <= W = NC), so warp 0
        // factors Ac = L L^T left-looking (lane p computes row k + p of
        // column k; warp-synchronous; measured faster than keeping the band
        // rows in registers and moving them by shuffles), then thread j
        // solves L L^T x = e_j for column j of the inverse.  Band storage
        // Lb[i][W - q] = L[i][i - q] and 1 / L[i][i] live in ub (free here);
        // the symmetrised probe is read from a1.
        constexpr int W = C::NC;
        float *__restrict__ Lb = reinterpret_cast<float *>(ub);
        float *__restrict__ invd = Lb + C::NI * (W + 1);
        const float *__restrict__ A1 = a1;
        // warp 0 factors column k while warp 1 computes row k - 1 of
        // X = L^-1 (which needs only the factor's rows up to k - 1), stored
        // transposed (XT[j][k] = X[k][j], row j of a0); a two-warp named
        // barrier per step orders them (measured faster than one warp
        // doing both, or X by columns after the factorisation)
        if (warp < 2) {
          float *__restrict__ XT = a0;
#pragma unroll 1
          for (int k = 0; k <= nI; ++k) {
            if (warp == 0) {
              if (k < nI) {
                const int i = k + lane;
                float sp = 0.0f;
                if (lane <= W && i < nI) {
                  sp = 0.5f * (A1[i * nI + k] + A1[k * nI + i]);
#pragma unroll
                  for (int q = 1; q <= W; ++q)
                    if (q <= W - lane && k - q >= 0) sp = fmaf(-Lb[i * (W + 1) + W - lane - q], Lb[k * (W + 1) + W - q], sp);
                }
                const float piv = __shfl_sync(0xffffffffu, sp, 0);
                const float id = piv > 0.0f ? rsqrtf(piv) : 0.0f;  // a lost pivot drops that coarse mode
                if (lane == 0) {
                  Lb[k * (W + 1) + W] = piv * id;
                  invd[k] = id;
                } else if (lane <= W && i < nI) {
                  Lb[i * (W + 1) + W - lane] = sp * id;
                }
              }
            } else {
              const int kk = k - 1;
              if (kk >= 0) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                  const int j = lane + 32 * h;
                  if (j < nI) {
                    float sx = kk == j ? 1.0f : 0.0f;
#pragma unroll
                    for (int q = W; q >= 1; --q)  // newest term last
                      if (kk - q >= 0) sx = fmaf(-Lb[kk * (W + 1) + W - q], XT[j * nI + kk - q], sx);
                    XT[j * nI + kk] = sx * invd[kk];
                  }
                }
              }
            }
            asm volatile("bar.sync 1, 64;" ::: "memory");  // warps 0 and 1, same count in both
          }
        }
        __syncthreads();
        // Ac^-1 = X^T X into a1 (the probe is no longer needed): entry (i, j),
        // i >= j, is the dot product of rows i and j of a0 from column i on
        {
          const int ntri = nI * (nI + 1) / 2;
          for (int e = tid; e < ntri; e += NT) {
            int i = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
            while (i > 0 && i * (i + 1) / 2 > e) --i;
            while ((i + 1) * (i + 2) / 2 <= e) ++i;
            const int j = e - i * (i + 1) / 2;
            const float *xi = a0 + i * nI, *xj = a0 + j * nI;
            float acc = 0.0f;
            for (int k = i; k < nI; ++k) acc = fmaf(xi[k], xj[k], acc);
            a1[i * nI + j] = acc;
            a1[j * nI + i] = acc;
          }
        }
        __syncthreads();
        Aci = a1;
      }
    }

    const double tol2 = p.tol * p.tol;
    const float itol2 = p.inner_tol * p.inner_tol;
    int total_iters[4] = {0, 0, 0, 0};
    int ref = 0;
    int buf = 0;
    // lane-parallel 4-value block sum (every warp ends with the totals)
    auto block_sum4 = [&](float (&v)[4]) {
      const float t = warp_transpose_reduce<4>(v, lane);
      if ((lane & 7) == 0) red32[buf][warp * 4 + (lane >> 3)] = t;
      __syncthreads();
      float s = 0.f;
      for (int i = lane; i < NW * 4; i += 32) s += red32[buf][i];
#pragma unroll
      for (int m = 4; m < 32; m <<= 1) s += shfl_xor_d(s, m);
#pragma unroll
      for (int r = 0; r < 4; ++r) v[r] = __shfl_sync(0xffffffffu, s, r);
      buf ^= 1;
    };
    for (;;) {
      // ---- true FP64 residual norm and convergence test
      double nup[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
      for (int s = 0; s < S; ++s)
        if (s < ns) {
#pragma unroll
          for (int r = 0; r < 4; ++r) nup[r] = fma(r64[s][r], r64[s][r], nup[r]);
        }
      warp_partials<4>(nup, red[0], warp, lane);
      __syncthreads();
      if (warp == 0) {
        const double t = warp_finish<4>(red[0], NW, lane);
        if (lane < 4) {
          cs.nu[lane] = t;
          if (!isfinite(t)) {
            cs.active[lane] = 0;
            cs.iters[lane] = -1;
          } else {
            cs.active[lane] = !(t <= tol2 * cs.bthr[lane]);
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
      float dv[S][4];
      if constexpr (M == 0) {
        // ---- inner FP32 CG on A~ d = r (active RHS only)
        float act[4];
  #pragma unroll
        for (int r = 0; r < 4; ++r) act[r] = cs.active[r] ? 1.0f : 0.0f;
        float rv[S][4], pv[S][4], qv[S][4];
        float rho[4] = {0.f, 0.f, 0.f, 0.f};
  #pragma unroll
        for (int s = 0; s < S; ++s) {
  #pragma unroll
          for (int r = 0; r < 4; ++r) {
            rv[s][r] = s < ns ? (float)r64[s][r] * sown[s] * act[r] : 0.0f;
            pv[s][r] = rv[s][r];
            dv[s][r] = 0.0f;
            qv[s][r] = 0.0f;
            rho[r] = fmaf(rv[s][r], rv[s][r], rho[r]);
          }
          if (s < ns) st4(v32, g0 + s * P, pv[s]);
        }
        block_sum4(rho);
        const float rho0[4] = {rho[0], rho[1], rho[2], rho[3]};
        // Inner target: the fixed relative reduction, but never deeper than the
        // outer goal needs (with a factor 10 margin): ||r|| <= 0.1 tol ||b||.
        float itol2r[4];
        bool iact[4];
  #pragma unroll
        for (int r = 0; r < 4; ++r) {
          iact[r] = act[r] > 0.0f && rho[r] > 0.0f;
          const double goal = cs.nu[r] > 0.0 ? 0.01 * tol2 * cs.bthr[r] / cs.nu[r] : 0.0;
          itol2r[r] = fmaxf(itol2, (float)fmin(goal, 0.25));
        }
        int iit = 0;
        for (;;) {
          if (!(iact[0] || iact[1] || iact[2] || iact[3]) || iit >= p.inner_maxit) break;
          ++iit;
          // q = A~ p on the strip.  Own-column neighbours come from registers
          // (halo rows from shared memory); each value of the two neighbour
          // columns is loaded once and scattered into the (up to three) rows
          // that couple to it.
          float sg[4] = {0.f, 0.f, 0.f, 0.f};
  #pragma unroll
          for (int s = 0; s < S; ++s)
  #pragma unroll
            for (int r = 0; r < 4; ++r) qv[s][r] = pv[s][r];
          if (ns > 0) {
            float t4[4];
            ld4(v32, g0 - P, t4);  // row below the strip
  #pragma unroll
            for (int r = 0; r < 4; ++r) qv[0][r] = fmaf(cp.cS[0], t4[r], qv[0][r]);
  #pragma unroll
            for (int s = 0; s < S; ++s) {
              if (s < ns) {
                if (s > 0) {
  #pragma unroll
                  for (int r = 0; r < 4; ++r) qv[s][r] = fmaf(cp.cS[s], pv[s - 1][r], qv[s][r]);
                }
                if (s + 1 < ns) {
  #pragma unroll
                  for (int r = 0; r < 4; ++r) qv[s][r] = fmaf(cp.cN[s], pv[s + 1][r], qv[s][r]);
                } else {
                  ld4(v32, g0 + (s + 1) * P, t4);  // row above the strip
  #pragma unroll
                  for (int r = 0; r < 4; ++r) qv[s][r] = fmaf(cp.cN[s], t4[r], qv[s][r]);
                }
              }
            }
  #pragma unroll
            for (int t = -1; t <= S; ++t) {
              if (t <= ns) {
                ld4(v32, g0 + t * P - 1, t4);  // left column, row s0 + t
                if (t >= 1 && t - 1 < ns) {
  #pragma unroll
                  for (int r = 0; r < 4; ++r) qv[t - 1][r] = fmaf(cp.cNW[t - 1], t4[r], qv[t - 1][r]);
                }
                if (t >= 0 && t < ns) {
  #pragma unroll
                  for (int r = 0; r < 4; ++r) qv[t][r] = fmaf(cp.cW[t], t4[r], qv[t][r]);
                }
                if (t + 1 < ns && t + 1 < S) {
  #pragma unroll
                  for (int r = 0; r < 4; ++r) qv[t + 1][r] = fmaf(cp.cSW[t + 1], t4[r], qv[t + 1][r]);
                }
                ld4(v32, g0 + t * P + 1, t4);  // right column, row s0 + t
                if (t >= 1 && t - 1 < ns) {
  #pragma unroll
                  for (int r = 0; r < 4; ++r) qv[t - 1][r] = fmaf(cp.cNE[t - 1], t4[r], qv[t - 1][r]);
                }
                if (t >= 0 && t < ns) {
  #pragma unroll
                  for (int r = 0; r < 4; ++r) qv[t][r] = fmaf(cp.cE[t], t4[r], qv[t][r]);
                }
                if (t + 1 < ns && t + 1 < S) {
  #pragma unroll
                  for (int r = 0; r < 4; ++r) qv[t + 1][r] = fmaf(cp.cSE[t + 1], t4[r], qv[t + 1][r]);
                }
              }
            }
  #pragma unroll
            for (int s = 0; s < S; ++s)
  #pragma unroll
              for (int r = 0; r < 4; ++r) sg[r] = fmaf(pv[s][r], qv[s][r], sg[r]);
          }
          block_sum4(sg);
          float al[4];
  #pragma unroll
          for (int r = 0; r < 4; ++r) al[r] = (iact[r] && sg[r] > 0.f) ? rho[r] / sg[r] : 0.0f;
          float rp[4] = {0.f, 0.f, 0.f, 0.f};
  #pragma unroll
          for (int s = 0; s < S; ++s)
  #pragma unroll
            for (int r = 0; r < 4; ++r) {
              dv[s][r] = fmaf(al[r], pv[s][r], dv[s][r]);
              rv[s][r] = fmaf(-al[r], qv[s][r], rv[s][r]);
              rp[r] = fmaf(rv[s][r], rv[s][r], rp[r]);
            }
          block_sum4(rp);
          float be[4];
  #pragma unroll
          for (int r = 0; r < 4; ++r) {
            be[r] = 0.0f;
            if (iact[r]) {
              total_iters[r] += 1;
              if (!(rp[r] <= itol2r[r] * rho0[r]) && isfinite(rp[r])) {
                be[r] = rp[r] / rho[r];
                rho[r] = rp[r];
              } else {
                iact[r] = false;
              }
            }
          }
  #pragma unroll
          for (int s = 0; s < S; ++s) {
  #pragma unroll
            for (int r = 0; r < 4; ++r) pv[s][r] = fmaf(be[r], pv[s][r], rv[s][r]);
            if (s < ns) st4(v32, g0 + s * P, pv[s]);
          }
          __syncthreads();
        }

      } else {
        // ---- inner FP32 CG on A~ d = r preconditioned by z = P(A~) r, the
        // Chebyshev polynomial of degree M - 1 on [b / ratio, b] (M - 1
        // stencils exchanged through v32b / v32 alternately, no reductions)
        float act[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) act[r] = cs.active[r] ? 1.0f : 0.0f;
        float rv[S][4], pv[S][4], zv[S][4], ddv[S][4];
#pragma unroll
        for (int s = 0; s < S; ++s)
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            rv[s][r] = s < ns ? (float)r64[s][r] * sown[s] * act[r] : 0.0f;
            dv[s][r] = 0.0f;
          }
        // Chebyshev smoothing in residual form: zv += p(A~) e, e tracking the
        // residual of the added part (its last update only when need_res)
        auto smooth = [&](float (&e)[S][4], bool need_res) {
          float dd[S][4], yv[S][4];
#pragma unroll
          for (int s = 0; s < S; ++s)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
              dd[s][r] = e[s][r] * cheb_inv_theta;
              zv[s][r] += dd[s][r];
            }
#pragma unroll
          for (int k = 1; k < M; ++k) {
            pass(dd, yv);
#pragma unroll
            for (int s = 0; s < S; ++s)
#pragma unroll
              for (int r = 0; r < 4; ++r) {
                e[s][r] -= yv[s][r];
                dd[s][r] = fmaf(cheb_c1[k], dd[s][r], cheb_c2[k] * e[s][r]);
                zv[s][r] += dd[s][r];
              }
          }
          if (need_res) {
            pass(dd, yv);
#pragma unroll
            for (int s = 0; s < S; ++s)
#pragma unroll
              for (int r = 0; r < 4; ++r) e[s][r] -= yv[s][r];
          }
        };
        auto apply_prec = [&]() {
          if constexpr (CH > 0) {
            // z = B r: pre-smoothing, coarse correction, post-smoothing
            float e[S][4];
#pragma unroll
            for (int s = 0; s < S; ++s)
#pragma unroll
              for (int r = 0; r < 4; ++r) {
                e[s][r] = rv[s][r];
                zv[s][r] = 0.0f;
              }
            if (coarse) {
              smooth(e, true);
              float cr[S][4], yv[S][4];
              restrict_c(e);
              coarse_solve(cr);
              pass(cr, yv);
#pragma unroll
              for (int s = 0; s < S; ++s)
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                  zv[s][r] += cr[s][r];
                  e[s][r] -= yv[s][r];
                }
            }
            smooth(e, false);
          } else {
#pragma unroll
            for (int s = 0; s < S; ++s)
#pragma unroll
              for (int r = 0; r < 4; ++r) {
                zv[s][r] = rv[s][r] * cheb_inv_theta;
                ddv[s][r] = zv[s][r];
              }
#pragma unroll
            for (int k = 1; k < M; ++k) {
              // two buffers alternate (one barrier per step); with one buffer
              // (MINB >= 2, less shared memory) a second barrier orders the
              // reads of step k before the writes of step k + 1
              float *bufk = (MINB >= 2 || (k & 1) == 0) ? v32 : v32b;
              if (MINB >= 2 && k > 1) __syncthreads();
              strip_store<S>(bufk, g0, P, ns, zv);
              __syncthreads();
              float yv[S][4];
              strip_apply_x2<S>(bufk, g0, P, ns, cp, zv, yv);
#pragma unroll
              for (int s = 0; s < S; ++s)
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                  ddv[s][r] = fmaf(cheb_c1[k], ddv[s][r], cheb_c2[k] * (rv[s][r] - yv[s][r]));
                  zv[s][r] += ddv[s][r];
                }
            }
          }
        };
        auto dots_rz_rr = [&](float (&out)[8]) {
#pragma unroll
          for (int j = 0; j < 8; ++j) out[j] = 0.0f;
#pragma unroll
          for (int s = 0; s < S; ++s)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
              out[r] = fmaf(rv[s][r], zv[s][r], out[r]);
              out[4 + r] = fmaf(rv[s][r], rv[s][r], out[4 + r]);
            }
          block_sum_f<8, NW>(out, red32[buf], warp, lane);
          buf ^= 1;
        };
        apply_prec();
        float rzrr[8];
        dots_rz_rr(rzrr);
        float rho[4], rho0[4], itol2r[4];
        bool iact[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          rho[r] = rzrr[r];
          rho0[r] = rzrr[4 + r];
          iact[r] = act[r] > 0.0f && rho0[r] > 0.0f && rho[r] > 0.0f;
          const double goal = cs.nu[r] > 0.0 ? 0.01 * tol2 * cs.bthr[r] / cs.nu[r] : 0.0;
          itol2r[r] = fmaxf(itol2, (float)fmin(goal, 0.25));
        }
#pragma unroll
        for (int s = 0; s < S; ++s)
#pragma unroll
          for (int r = 0; r < 4; ++r) pv[s][r] = zv[s][r];
        int iit = 0;
        for (;;) {
          if (!(iact[0] || iact[1] || iact[2] || iact[3]) || iit >= p.inner_maxit) break;
          ++iit;
          // q = A~ p (p exchanged through v32; the two-level form alternates)
          float qv[S][4];
          if constexpr (CH > 0) {
            pass(pv, qv);
          } else {
            strip_store<S>(v32, g0, P, ns, pv);
            __syncthreads();
            strip_apply_x2<S>(v32, g0, P, ns, cp, pv, qv);
          }
          float sg[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
          for (int s = 0; s < S; ++s)
#pragma unroll
            for (int r = 0; r < 4; ++r) sg[r] = fmaf(pv[s][r], qv[s][r], sg[r]);
          block_sum_f<4, NW>(sg, red32[buf], warp, lane);
          buf ^= 1;
          float al[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) al[r] = (iact[r] && sg[r] > 0.f) ? rho[r] / sg[r] : 0.0f;
#pragma unroll
          for (int s = 0; s < S; ++s)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
              dv[s][r] = fmaf(al[r], pv[s][r], dv[s][r]);
              rv[s][r] = fmaf(-al[r], qv[s][r], rv[s][r]);
            }
          apply_prec();
          dots_rz_rr(rzrr);
          float be[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            be[r] = 0.0f;
            if (iact[r]) {
              total_iters[r] += 1;
              const float rr = rzrr[4 + r], rz = rzrr[r];
              if (!(rr <= itol2r[r] * rho0[r]) && isfinite(rr) && rz > 0.0f && sg[r] > 0.0f) {
                be[r] = rz / rho[r];
                rho[r] = rz;
              } else {
                iact[r] = false;
              }
            }
          }
#pragma unroll
          for (int s = 0; s < S; ++s)
#pragma unroll
            for (int r = 0; r < 4; ++r) pv[s][r] = fmaf(be[r], pv[s][r], zv[s][r]);
        }
        __syncthreads();  // last reads of v32 / v32b before the next writes
      }
      // ---- x += s d (FP64), new FP64 residual r = -(A phi)_I
#pragma unroll
      for (int s = 0; s < S; ++s)
        if (s < ns) {
          double xs[4];
          ld4(v64, g0 + s * P, xs);
#pragma unroll
          for (int r = 0; r < 4; ++r) xs[r] += f32_to_f64(dv[s][r] * sown[s]);
          st4(v64, g0 + s * P, xs);
        }
      __syncthreads();
#pragma unroll
      for (int s = 0; s < S; ++s)
        if (s < ns) {
          double y[4];
          stencil9_unscaled(c64, d64, v64, g0 + s * P, P, y);
#pragma unroll
          for (int r = 0; r < 4; ++r) r64[s][r] = -y[r];
        }
    }
    if (tid == 0) cs.refinements = ref;

    // ---------------- epilogue ----------------------------------------
    // interior: A phi = -r (the converged FP64 residual, in registers); M is
    // symmetric, so 10 of its entries are accumulated
    double acc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = 0.0;
#pragma unroll
    for (int s = 0; s < S; ++s)
      if (s < ns) {
        double ph[4], y[4];
        ld4(v64, g0 + s * P, ph);
#pragma unroll
        for (int r = 0; r < 4; ++r) y[r] = -r64[s][r];
        epilogue_node_sym(p, cs, N, ix, s0 + s, ph, y, acc);
      }
    // boundary rows: stencil of the unconstrained matrix
    for (int k = tid; k < 4 * N; k += NT) {
      int bx, by;
      boundary_node(k, N, bx, by);
      const int g = (by + 1) * P + bx + 1;
      double y[4], ph[4];
      stencil9_unscaled(c64, d64, v64, g, P, y);
      ld4(v64, g, ph);
      epilogue_node_sym(p, cs, N, bx, by, ph, y, acc);
    }
    write_basis<NT, false>(p, cell, N, v64, d64, tid);
    __syncthreads();  // v32 is reused for the 32-value partials below
    epilogue_finish_sym<NT>(p, cs, cell, acc, reinterpret_cast<double *>(v32), total_iters, tid);
  }
}

// ===========================================================================
// Energy norms of basis functions against a reference basis
// ===========================================================================
// err[cell][i] = ||phi_i - ref_i||_A and nrm[cell][i] = ||ref_i||_A with A the
// cell's fine Q1 stiffness over all nodes (the unconstrained diffusion_matrix
// of diffusion_problem_basis.tpp:159-242), summed element by element:
// e^T A e = sum_c e_c^T K_c e_c.  For a converged ref, nrm^2 = M_ii.  Bases
// in the basis-output layout ([cell][4][(N+1)^2], lexicographic nodes).
template <int NT>
__global__ void __launch_bounds__(NT)
msfem2d_energy_kernel(const KernelParams p, const double *__restrict__ basis,
                      const double *__restrict__ ref, double *__restrict__ err,
                      double *__restrict__ nrm) {
  constexpr int NW = NT / 32;
  __shared__ CellShared2D cs;
  __shared__ double red[NW * 8];
  __shared__ int bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int cell = blockIdx.x; cell < p.n_cells; cell += gridDim.x) {
    const int N = p.n_fine ? p.n_fine[cell] : p.n_fine_uniform;
    if (tid == 0) bad = 0;
    const int st = cell_geometry2d<MSFEM_MAX_N_2D>(p, cs, cell, N, tid);
    double acc[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i] = 0.0;
    if (st == MSFEM_CELL_CONVERGED) {
      const int n = N + 1, nn = n * n;
      const int64_t off = p.basis_offset ? p.basis_offset[cell] : (int64_t)cell * 4 * nn;
      const double *a = basis + off, *r = ref + off;
      const double *tab = nullptr;
      if (p.coef_kind == MSFEM_COEF_TABULATED)
        tab = p.qp_values + (p.qp_offset ? p.qp_offset[cell] : (int64_t)cell * p.ncomp * 4 * N * N);
      const bool need_x = p.coef_kind != MSFEM_COEF_TABULATED && p.coef_kind != MSFEM_COEF_CONSTANT;
      for (int fc = tid; fc < N * N; fc += NT) {
        const int cx = fc % N, cy = fc / N;
        double Kd[4], Ko[6];
        if (!element2d(p, cs, tab, N, cx, cy, need_x, Kd, Ko)) bad = 1;
        const int k0 = cy * n + cx;
        const int kk[4] = {k0, k0 + 1, k0 + n, k0 + n + 1};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          double e[4], v[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            v[j] = r[(int64_t)i * nn + kk[j]];
            e[j] = a[(int64_t)i * nn + kk[j]] - v[j];
          }
          double qe = Kd[0] * e[0] * e[0] + Kd[1] * e[1] * e[1] + Kd[2] * e[2] * e[2] + Kd[3] * e[3] * e[3];
          double qv = Kd[0] * v[0] * v[0] + Kd[1] * v[1] * v[1] + Kd[2] * v[2] * v[2] + Kd[3] * v[3] * v[3];
          qe += 2.0 * (Ko[0] * e[0] * e[1] + Ko[1] * e[0] * e[2] + Ko[2] * e[0] * e[3] +
                       Ko[3] * e[1] * e[2] + Ko[4] * e[1] * e[3] + Ko[5] * e[2] * e[3]);
          qv += 2.0 * (Ko[0] * v[0] * v[1] + Ko[1] * v[0] * v[2] + Ko[2] * v[0] * v[3] +
                       Ko[3] * v[1] * v[2] + Ko[4] * v[1] * v[3] + Ko[5] * v[2] * v[3]);
          acc[i] += qe;
          acc[4 + i] += qv;
        }
      }
    }
    warp_partials<8>(acc, red, warp, lane);
    __syncthreads();
    if (warp == 0) {
      const double s = warp_finish<8>(red, NW, lane);
      if (lane < 8) {
        double out = sqrt(fmax(s, 0.0));
        if (st != MSFEM_CELL_CONVERGED || bad || !isfinite(s)) out = qnan();
        (lane < 4 ? err : nrm)[(int64_t)cell * 4 + (lane & 3)] = out;
      }
    }
    __syncthreads();
  }
}

}  // namespace msfem
