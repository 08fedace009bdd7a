/*
 * msfem_oracle.c -- CPU FP64 restatement of the reference's per-coarse-cell
 * multiscale basis computation.  TEST INFRASTRUCTURE ONLY (see msfem_oracle.h
 * for scope, citations and the parity status: unpinned against reference
 * outputs, pinned against analytic known answers).
 *
 * Plain C11 + pthreads, portable (no intrinsics, no -march flags).
 */
#include "msfem_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* include/coefficients/coefficients.h:21 -- the reference's (mistyped) pi. */
static const double OC_PI_D = 3.14592653509793218403;
static const double OC_PI = 3.14159265358979323846;

#define MAXD 3

/* ------------------------------------------------------------------------ */
/* geometry                                                                  */
/* ------------------------------------------------------------------------ */

static int cell_n(const oc_batch *b, int32_t cell) {
  return b->n_fine_per_cell ? b->n_fine_per_cell[cell] : b->n_fine;
}

static int ipow(int a, int e) {
  int r = 1;
  while (e-- > 0) r *= a;
  return r;
}

/* Multilinear map of the coarse cell: corners in deal.II vertex order
 * (v = vx + 2 vy + 4 vz).  GridGenerator::general_cell + refine_global on a
 * straight-sided cell (diffusion_problem_basis.tpp:94-98) places every fine
 * vertex at this map of the uniform lattice. */
static void coarse_map(int dim, const double *corners, const double *t,
                       double *x) {
  int nv = 1 << dim;
  for (int c = 0; c < dim; ++c) x[c] = 0.0;
  for (int v = 0; v < nv; ++v) {
    double w = 1.0;
    for (int a = 0; a < dim; ++a) w *= ((v >> a) & 1) ? t[a] : 1.0 - t[a];
    for (int c = 0; c < dim; ++c) x[c] += w * corners[v * dim + c];
  }
}

static void node_pos(int dim, const double *corners, int N, const int *ijk,
                     double *x) {
  double t[MAXD];
  for (int a = 0; a < dim; ++a) t[a] = (double)ijk[a] / (double)N;
  coarse_map(dim, corners, t, x);
}

/* ------------------------------------------------------------------------ */
/* coefficients                                                              */
/* ------------------------------------------------------------------------ */

typedef struct sphere_grid {
  int G;
  double lo[MAXD], h;
  int *start; /* G^d + 1 */
  int *ids;
} sphere_grid;

static pthread_mutex_t g_sphere_mu = PTHREAD_MUTEX_INITIALIZER;
static sphere_grid g_sg;
static const double *g_sg_src = NULL;
static int g_sg_n = 0, g_sg_dim = 0;

static void sphere_grid_build(int dim, const double *sp, int n) {
  double rmax = 0.0;
  for (int s = 0; s < n; ++s) if (sp[4 * s + 3] > rmax) rmax = sp[4 * s + 3];
  double h = fmax(2.0 * rmax, 1e-3);
  int G = (int)ceil(1.0 / h);
  if (G < 1) G = 1;
  if (G > 256) G = 256;
  h = 1.0 / G;
  int ncell = ipow(G, dim);
  int *cnt = calloc((size_t)ncell + 1, sizeof(int));
  for (int pass = 0; pass < 2; ++pass) {
    for (int s = 0; s < n; ++s) {
      int lo[MAXD] = {0, 0, 0}, hi[MAXD] = {0, 0, 0};
      for (int a = 0; a < dim; ++a) {
        double c = sp[4 * s + a], r = sp[4 * s + 3];
        lo[a] = (int)floor((c - r) / h);
        hi[a] = (int)floor((c + r) / h);
        if (lo[a] < 0) lo[a] = 0;
        if (hi[a] > G - 1) hi[a] = G - 1;
      }
      for (int k = lo[2]; k <= hi[2]; ++k)
        for (int j = lo[1]; j <= hi[1]; ++j)
          for (int i = lo[0]; i <= hi[0]; ++i) {
            int g = i + G * (j + (dim == 3 ? G * k : 0));
            if (pass == 0) cnt[g + 1]++;
            else g_sg.ids[cnt[g]++] = s;
          }
    }
    if (pass == 0) {
      for (int g = 0; g < ncell; ++g) cnt[g + 1] += cnt[g];
      free(g_sg.start);
      free(g_sg.ids);
      g_sg.start = malloc(((size_t)ncell + 1) * sizeof(int));
      memcpy(g_sg.start, cnt, ((size_t)ncell + 1) * sizeof(int));
      g_sg.ids = malloc((size_t)(cnt[ncell] > 0 ? cnt[ncell] : 1) * sizeof(int));
    }
  }
  free(cnt);
  g_sg.G = G;
  g_sg.h = h;
  g_sg_src = sp;
  g_sg_n = n;
  g_sg_dim = dim;
}

static int inside_sphere(int dim, const double *sp, int n, const double *x) {
  int G = g_sg.G, idx[MAXD] = {0, 0, 0};
  for (int a = 0; a < dim; ++a) {
    int i = (int)floor(x[a] / g_sg.h);
    if (i < 0) i = 0;
    if (i > G - 1) i = G - 1;
    idx[a] = i;
  }
  int g = idx[0] + G * (idx[1] + (dim == 3 ? G * idx[2] : 0));
  (void)n;
  for (int e = g_sg.start[g]; e < g_sg.start[g + 1]; ++e) {
    const double *s = sp + 4 * g_sg.ids[e];
    double d2 = 0.0;
    for (int a = 0; a < dim; ++a) d2 += (x[a] - s[a]) * (x[a] - s[a]);
    if (d2 <= s[3] * s[3]) return 1;
  }
  return 0;
}

static void sym_to_full(int dim, const double *c, double *A) {
  if (dim == 2) {
    A[0] = c[0]; A[1] = c[1]; A[2] = c[1]; A[3] = c[2];
  } else {
    A[0] = c[0]; A[1] = c[1]; A[2] = c[2];
    A[3] = c[1]; A[4] = c[3]; A[5] = c[4];
    A[6] = c[2]; A[7] = c[4]; A[8] = c[5];
  }
}

static double fourier_field(const oc_coef *c, int dim, int f, const double *x) {
  double g = 0.0;
  for (int m = 0; m < c->n_modes; ++m) {
    const double *md = c->modes + ((size_t)f * c->n_modes + m) * 5;
    double ph = md[0] * x[0] + md[1] * x[1] + (dim == 3 ? md[2] * x[2] : 0.0) + md[4];
    g += md[3] * cos(ph);
  }
  return g;
}

/* MatrixCoeff<dim> rotation, matrix_coeff.tpp:17-41 (alpha = PI_D/3,
 * beta = PI_D/6, gamma = PI_D/4, matrix_coeff.hpp:48). */
static void reference_rotation(int dim, double *R) {
  const double al = OC_PI_D / 3, be = OC_PI_D / 6, ga = OC_PI_D / 4;
  if (dim == 2) {
    R[0] = cos(al); R[1] = sin(al);
    R[2] = -sin(al); R[3] = cos(al);
  } else {
    R[0] = cos(al) * cos(ga) - sin(al) * cos(be) * sin(ga);
    R[1] = -cos(al) * sin(ga) - sin(al) * cos(be) * cos(ga);
    R[2] = sin(al) * sin(be);
    R[3] = sin(al) * cos(ga) + cos(al) * cos(be) * sin(ga);
    R[4] = -sin(al) * sin(ga) + cos(al) * cos(be) * cos(ga);
    R[5] = -cos(al) * sin(be);
    R[6] = sin(be) * sin(ga);
    R[7] = sin(be) * cos(ga);
    R[8] = cos(be);
  }
}

/* A = R D R^T (row-major, d x d). */
static void rotate(int dim, const double *R, const double *D, double *A) {
  double T[9];
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j) {
      double s = 0.0;
      for (int k = 0; k < dim; ++k) s += R[i * dim + k] * D[k * dim + j];
      T[i * dim + j] = s;
    }
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j) {
      double s = 0.0;
      for (int k = 0; k < dim; ++k) s += T[i * dim + k] * R[j * dim + k];
      A[i * dim + j] = s;
    }
}

void oc_coef_eval(const oc_batch *b, int32_t cell, int32_t fc, int32_t q,
                  const double *x, double *A) {
  const oc_coef *c = &b->coef;
  const int dim = b->dim;
  for (int i = 0; i < dim * dim; ++i) A[i] = 0.0;
  switch (c->kind) {
  case OC_COEF_CONSTANT:
    sym_to_full(dim, c->params, A);
    break;
  case OC_COEF_REFERENCE: {
    /* matrix_coeff.tpp:66-91: diagonal c(x) from x and y only, then R c R^T */
    const int k = 57;
    const double scale = 0.9999;
    double v = 1.0 * (1.0 - scale * (0.5 * sin(2 * OC_PI_D * k * x[0]) +
                                     0.5 * sin(2 * OC_PI_D * k * x[1])));
    double D[9] = {0}, R[9];
    for (int d = 0; d < dim; ++d) D[d * dim + d] = v;
    reference_rotation(dim, R);
    rotate(dim, R, D, A);
    break;
  }
  case OC_COEF_SINSIN: {
    double amp = c->params[0], eps = c->params[1];
    double s = sin(2 * OC_PI * x[0] / eps) * sin(2 * OC_PI * x[1] / eps);
    if (dim == 3) s *= sin(2 * OC_PI * x[2] / eps);
    double v = 1.0 + amp * s;
    for (int d = 0; d < dim; ++d) A[d * dim + d] = v;
    break;
  }
  case OC_COEF_FOURIER: {
    if (dim == 2) {
      double g1 = fourier_field(c, dim, 0, x), g2 = fourier_field(c, dim, 1, x);
      double th = fourier_field(c, dim, 2, x);
      double R[4] = {cos(th), -sin(th), sin(th), cos(th)};
      double D[4] = {exp(g1), 0.0, 0.0, exp(g2)};
      rotate(2, R, D, A);
    } else {
      double v = exp(fourier_field(c, dim, 0, x));
      for (int d = 0; d < dim; ++d) A[d * dim + d] = v;
    }
    break;
  }
  case OC_COEF_SPHERES: {
    double v = inside_sphere(dim, c->spheres, c->n_spheres, x) ? c->params[0] : 1.0;
    for (int d = 0; d < dim; ++d) A[d * dim + d] = v;
    break;
  }
  case OC_COEF_TABULATED: {
    int N = cell_n(b, cell);
    int nq = 1 << dim, nfc = ipow(N, dim);
    int64_t base = c->qp_offset ? c->qp_offset[cell]
                                : (int64_t)cell * c->ncomp * nq * nfc;
    double comp[6];
    for (int k = 0; k < c->ncomp; ++k)
      comp[k] = c->qp_values[base + ((int64_t)k * nq + q) * nfc + fc];
    if (c->ncomp == 1) {
      for (int d = 0; d < dim; ++d) A[d * dim + d] = comp[0];
    } else {
      sym_to_full(dim, comp, A);
    }
    break;
  }
  default:
    break;
  }
}

/* ------------------------------------------------------------------------ */
/* BasisQ1, basis_q1.tpp:26-158                                              */
/* ------------------------------------------------------------------------ */

/* monomials {1,x,y,xy} / {1,x,y,z,xy,yz,xz,xyz}, basis_q1.tpp:29-32, 53-60 */
static void monomials(int dim, const double *x, double *m) {
  if (dim == 2) {
    m[0] = 1; m[1] = x[0]; m[2] = x[1]; m[3] = x[0] * x[1];
  } else {
    m[0] = 1; m[1] = x[0]; m[2] = x[1]; m[3] = x[2];
    m[4] = x[0] * x[1]; m[5] = x[1] * x[2]; m[6] = x[0] * x[2];
    m[7] = x[0] * x[1] * x[2];
  }
}

/* Gauss-Jordan inverse with partial pivoting (n <= 8). */
static int invert(int n, double *a, double *inv) {
  double w[8][16];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 2 * n; ++j)
      w[i][j] = j < n ? a[i * n + j] : (j - n == i ? 1.0 : 0.0);
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int r = col + 1; r < n; ++r)
      if (fabs(w[r][col]) > fabs(w[piv][col])) piv = r;
    if (w[piv][col] == 0.0) return -1;
    if (piv != col)
      for (int j = 0; j < 2 * n; ++j) {
        double t = w[col][j]; w[col][j] = w[piv][j]; w[piv][j] = t;
      }
    double d = w[col][col];
    for (int j = 0; j < 2 * n; ++j) w[col][j] /= d;
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      double f = w[r][col];
      if (f != 0.0)
        for (int j = 0; j < 2 * n; ++j) w[r][j] -= f * w[col][j];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) inv[i * n + j] = w[i][j + n];
  return 0;
}

/* Coefficients of the 2^d interpolating polynomials: coef[m][i] (column i =
 * basis i), as coeff_matrix = inverse(point_matrix).  Unless raw_monomials
 * is set, the monomials are taken in the translated, scaled coordinates
 * x' = (x - v0)/H, which span the same polynomial space (so the interpolant
 * is the same function) with a far better conditioned Vandermonde matrix. */
typedef struct q1data {
  double coef[64];
  double shift[MAXD], scale;
} q1data;

static void q1_setup(const oc_batch *b, int32_t cell, q1data *q) {
  const int dim = b->dim, nv = 1 << dim;
  const double *cr = b->corners + (size_t)cell * nv * dim;
  double P[64];
  if (b->raw_monomials) {
    for (int a = 0; a < dim; ++a) q->shift[a] = 0.0;
    q->scale = 1.0;
  } else {
    double H = 0.0;
    for (int a = 0; a < dim; ++a) q->shift[a] = cr[a];
    for (int v = 1; v < nv; ++v)
      for (int a = 0; a < dim; ++a) H = fmax(H, fabs(cr[v * dim + a] - cr[a]));
    q->scale = H > 0 ? H : 1.0;
  }
  for (int v = 0; v < nv; ++v) {
    double xp[MAXD];
    for (int a = 0; a < dim; ++a) xp[a] = (cr[v * dim + a] - q->shift[a]) / q->scale;
    monomials(dim, xp, P + v * nv);
  }
  invert(nv, P, q->coef);
}

static void q1_eval(int dim, const q1data *q, const double *x, double *out) {
  int nv = 1 << dim;
  double xp[MAXD], m[8];
  for (int a = 0; a < dim; ++a) xp[a] = (x[a] - q->shift[a]) / q->scale;
  monomials(dim, xp, m);
  for (int i = 0; i < nv; ++i) {
    double s = 0.0;
    for (int k = 0; k < nv; ++k) s += q->coef[k * nv + i] * m[k];
    out[i] = s;
  }
}

void oc_basis_q1(const oc_batch *b, int32_t cell, const double *x, double *out) {
  q1data q;
  q1_setup(b, cell, &q);
  q1_eval(b->dim, &q, x, out);
}

/* ------------------------------------------------------------------------ */
/* assembly, diffusion_problem_basis.tpp:159-242                             */
/* ------------------------------------------------------------------------ */

static void qgauss2(double *g) {
  g[0] = 0.5 - 0.5 / sqrt(3.0);
  g[1] = 0.5 + 0.5 / sqrt(3.0);
}

/* Gauss point q of fine cell fc (physical position) -- used for tabulation. */
static void fine_cell_vertices(int dim, const double *corners, int N,
                               const int *cidx, double *V) {
  int nv = 1 << dim;
  for (int k = 0; k < nv; ++k) {
    int ijk[MAXD];
    for (int a = 0; a < dim; ++a) ijk[a] = cidx[a] + ((k >> a) & 1);
    node_pos(dim, corners, N, ijk, V + k * dim);
  }
}

/* Shape values/gradients of the reference Q1 element at xi. */
static void q1_shape(int dim, const double *xi, double *psi, double *dpsi) {
  int nv = 1 << dim;
  for (int k = 0; k < nv; ++k) {
    double v = 1.0;
    for (int a = 0; a < dim; ++a) v *= ((k >> a) & 1) ? xi[a] : 1.0 - xi[a];
    psi[k] = v;
    for (int a = 0; a < dim; ++a) {
      double d = ((k >> a) & 1) ? 1.0 : -1.0;
      for (int c = 0; c < dim; ++c)
        if (c != a) d *= ((k >> c) & 1) ? xi[c] : 1.0 - xi[c];
      dpsi[k * dim + a] = d;
    }
  }
}

static double det_inv(int dim, const double *J, double *Ji) {
  if (dim == 2) {
    double det = J[0] * J[3] - J[1] * J[2];
    Ji[0] = J[3] / det; Ji[1] = -J[1] / det;
    Ji[2] = -J[2] / det; Ji[3] = J[0] / det;
    return det;
  }
  double c00 = J[4] * J[8] - J[5] * J[7];
  double c01 = J[5] * J[6] - J[3] * J[8];
  double c02 = J[3] * J[7] - J[4] * J[6];
  double det = J[0] * c00 + J[1] * c01 + J[2] * c02;
  Ji[0] = c00 / det;
  Ji[1] = (J[2] * J[7] - J[1] * J[8]) / det;
  Ji[2] = (J[1] * J[5] - J[2] * J[4]) / det;
  Ji[3] = c01 / det;
  Ji[4] = (J[0] * J[8] - J[2] * J[6]) / det;
  Ji[5] = (J[2] * J[3] - J[0] * J[5]) / det;
  Ji[6] = c02 / det;
  Ji[7] = (J[1] * J[6] - J[0] * J[7]) / det;
  Ji[8] = (J[0] * J[4] - J[1] * J[3]) / det;
  return det;
}

static int stencil_slot(int dim, const int *off) {
  int s = 0, m = 1;
  for (int a = 0; a < dim; ++a) {
    s += (off[a] + 1) * m;
    m *= 3;
  }
  return s;
}

int oc_assemble_cell(const oc_batch *b, int32_t cell, double *st, double *bl) {
  const int dim = b->dim, nv = 1 << dim, N = cell_n(b, cell), n = N + 1;
  const int nn = ipow(n, dim), ns = ipow(3, dim), nfc = ipow(N, dim);
  const double *cr = b->corners + (size_t)cell * nv * dim;
  memset(st, 0, sizeof(double) * (size_t)nn * ns);
  memset(bl, 0, sizeof(double) * (size_t)nn);
  double g[2];
  qgauss2(g);
  const double w = 1.0 / nv; /* QGauss(2) weight per point on [0,1]^d */
  const double *fq_cell = NULL;
  if (b->f_qp_values) {
    int64_t off = 0;
    if (b->f_qp_offset) off = b->f_qp_offset[cell];
    else for (int c = 0; c < cell; ++c) off += (int64_t)nv * ipow(cell_n(b, c), dim);
    fq_cell = b->f_qp_values + off;
  }
  for (int fc = 0; fc < nfc; ++fc) {
    int cidx[MAXD] = {fc % N, (fc / N) % N, dim == 3 ? fc / (N * N) : 0};
    double V[8 * MAXD];
    fine_cell_vertices(dim, cr, N, cidx, V);
    double K[64] = {0}, be[8] = {0};
    for (int q = 0; q < nv; ++q) {
      double xi[MAXD], psi[8], dpsi[8 * MAXD];
      for (int a = 0; a < dim; ++a) xi[a] = g[(q >> a) & 1];
      q1_shape(dim, xi, psi, dpsi);
      double J[9] = {0}, Ji[9], xq[MAXD] = {0, 0, 0};
      for (int k = 0; k < nv; ++k)
        for (int a = 0; a < dim; ++a) {
          xq[a] += psi[k] * V[k * dim + a];
          for (int c = 0; c < dim; ++c) J[a * dim + c] += V[k * dim + a] * dpsi[k * dim + c];
        }
      double det = det_inv(dim, J, Ji);
      double JxW = w * fabs(det);
      double A[9];
      oc_coef_eval(b, cell, fc, q, xq, A);
      /* f at this Gauss point: RightHandSide::value_list (right_hand_side.tpp:27-40) */
      const double fq_val = fq_cell ? fq_cell[(size_t)q * nfc + fc] : b->f_value;
      /* physical gradients J^{-T} grad_ref */
      double G[8 * MAXD];
      for (int k = 0; k < nv; ++k)
        for (int a = 0; a < dim; ++a) {
          double s = 0.0;
          for (int c = 0; c < dim; ++c) s += Ji[c * dim + a] * dpsi[k * dim + c];
          G[k * dim + a] = s;
        }
      for (int i = 0; i < nv; ++i) {
        double AG[MAXD];
        for (int a = 0; a < dim; ++a) {
          double s = 0.0;
          for (int c = 0; c < dim; ++c) s += A[a * dim + c] * G[i * dim + c];
          AG[a] = s;
        }
        for (int j = 0; j < nv; ++j) {
          double s = 0.0;
          for (int a = 0; a < dim; ++a) s += G[j * dim + a] * AG[a];
          K[j * nv + i] += s * JxW; /* A symmetric: grad_j . A grad_i */
        }
        be[i] += psi[i] * fq_val * JxW;
      }
    }
    for (int i = 0; i < nv; ++i) {
      int ni[MAXD];
      for (int a = 0; a < dim; ++a) ni[a] = cidx[a] + ((i >> a) & 1);
      int gi = ni[0] + n * (ni[1] + (dim == 3 ? n * ni[2] : 0));
      for (int j = 0; j < nv; ++j) {
        int off[MAXD];
        for (int a = 0; a < dim; ++a) off[a] = ((j >> a) & 1) - ((i >> a) & 1);
        st[(size_t)gi * ns + stencil_slot(dim, off)] += K[i * nv + j];
      }
      bl[gi] += be[i];
    }
  }
  return 0;
}

int oc_tabulate(const oc_batch *b, int32_t ncomp, double *out) {
  const int dim = b->dim, nv = 1 << dim;
  double g[2];
  qgauss2(g);
  int64_t base = 0;
  if (b->coef.kind == OC_COEF_SPHERES) {
    pthread_mutex_lock(&g_sphere_mu);
    if (g_sg_src != b->coef.spheres || g_sg_n != b->coef.n_spheres || g_sg_dim != dim)
      sphere_grid_build(dim, b->coef.spheres, b->coef.n_spheres);
    pthread_mutex_unlock(&g_sphere_mu);
  }
  for (int cell = 0; cell < b->n_cells; ++cell) {
    const int N = cell_n(b, cell), nfc = ipow(N, dim);
    const double *cr = b->corners + (size_t)cell * nv * dim;
    for (int fc = 0; fc < nfc; ++fc) {
      int cidx[MAXD] = {fc % N, (fc / N) % N, dim == 3 ? fc / (N * N) : 0};
      double V[8 * MAXD];
      fine_cell_vertices(dim, cr, N, cidx, V);
      for (int q = 0; q < nv; ++q) {
        double xi[MAXD], psi[8], dpsi[8 * MAXD], xq[MAXD] = {0, 0, 0}, A[9];
        for (int a = 0; a < dim; ++a) xi[a] = g[(q >> a) & 1];
        q1_shape(dim, xi, psi, dpsi);
        for (int k = 0; k < nv; ++k)
          for (int a = 0; a < dim; ++a) xq[a] += psi[k] * V[k * dim + a];
        oc_coef_eval(b, cell, fc, q, xq, A);
        double comp[6];
        if (ncomp == 1) comp[0] = A[0];
        else if (dim == 2) { comp[0] = A[0]; comp[1] = A[1]; comp[2] = A[3]; }
        else { comp[0] = A[0]; comp[1] = A[1]; comp[2] = A[2];
               comp[3] = A[4]; comp[4] = A[5]; comp[5] = A[8]; }
        for (int k = 0; k < ncomp; ++k)
          out[base + ((int64_t)k * nv + q) * nfc + fc] = comp[k];
      }
    }
    base += (int64_t)ncomp * nv * nfc;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* local solves                                                              */
/* ------------------------------------------------------------------------ */

typedef struct local_sys {
  int dim, N, n, nn, ns, nI;
  int *node_of;   /* interior unknown -> node */
  int *unk_of;    /* node -> interior unknown or -1 */
  const double *st;
} local_sys;

static void local_sys_init(local_sys *L, int dim, int N, const double *st) {
  L->dim = dim; L->N = N; L->n = N + 1;
  L->nn = ipow(L->n, dim); L->ns = ipow(3, dim);
  L->nI = ipow(N - 1, dim);
  L->st = st;
  L->node_of = malloc(sizeof(int) * (size_t)(L->nI > 0 ? L->nI : 1));
  L->unk_of = malloc(sizeof(int) * (size_t)L->nn);
  int u = 0;
  for (int g = 0; g < L->nn; ++g) {
    int ix = g % L->n, iy = (g / L->n) % L->n, iz = dim == 3 ? g / (L->n * L->n) : 1;
    int inter = ix > 0 && ix < N && iy > 0 && iy < N && (dim == 2 || (iz > 0 && iz < N));
    L->unk_of[g] = inter ? u : -1;
    if (inter) L->node_of[u++] = g;
  }
}

static void local_sys_free(local_sys *L) {
  free(L->node_of);
  free(L->unk_of);
}

static int nbr(const local_sys *L, int g, int s) {
  int off[MAXD], m = s;
  for (int a = 0; a < L->dim; ++a) { off[a] = m % 3 - 1; m /= 3; }
  int ix = g % L->n + off[0], iy = (g / L->n) % L->n + off[1];
  int iz = L->dim == 3 ? g / (L->n * L->n) + off[2] : 0;
  if (ix < 0 || ix >= L->n || iy < 0 || iy >= L->n || iz < 0 || iz >= L->n) return -1;
  return ix + L->n * (iy + L->n * iz);
}

/* y = A_full x over all nodes (unconstrained matrix, as diffusion_matrix.vmult) */
static void spmv_full(const local_sys *L, const double *x, double *y) {
  for (int g = 0; g < L->nn; ++g) {
    double s = 0.0;
    for (int k = 0; k < L->ns; ++k) {
      double a = L->st[(size_t)g * L->ns + k];
      if (a == 0.0) continue;
      int h = nbr(L, g, k);
      if (h >= 0) s += a * x[h];
    }
    y[g] = s;
  }
}

/* Banded Cholesky of A_II in lexicographic interior order; solves nr RHS. */
static int solve_direct(const local_sys *L, int nr, double *rhs /* [nr][nI] in/out */) {
  const int nI = L->nI, m = L->N - 1;
  if (nI == 0) return 0;
  const int bw = L->dim == 2 ? m + 1 : m * m + m + 1;
  double *Lb = calloc((size_t)nI * (bw + 1), sizeof(double)); /* Lb[i][i-j] */
#define LB(i, j) Lb[(size_t)(i) * (bw + 1) + ((i) - (j))]
  for (int u = 0; u < nI; ++u) {
    int g = L->node_of[u];
    for (int k = 0; k < L->ns; ++k) {
      int h = nbr(L, g, k);
      if (h < 0) continue;
      int v = L->unk_of[h];
      if (v < 0 || v > u) continue;
      LB(u, v) = L->st[(size_t)g * L->ns + k];
    }
  }
  for (int j = 0; j < nI; ++j) {
    int k0 = j - bw > 0 ? j - bw : 0;
    double s = LB(j, j);
    for (int k = k0; k < j; ++k) s -= LB(j, k) * LB(j, k);
    if (!(s > 0.0)) { free(Lb); return -1; }
    double d = sqrt(s);
    LB(j, j) = d;
    int i1 = j + bw < nI - 1 ? j + bw : nI - 1;
    for (int i = j + 1; i <= i1; ++i) {
      int kk = i - bw > 0 ? i - bw : 0;
      double t = LB(i, j);
      for (int k = kk; k < j; ++k) t -= LB(i, k) * LB(j, k);
      LB(i, j) = t / d;
    }
  }
  for (int r = 0; r < nr; ++r) {
    double *y = rhs + (size_t)r * nI;
    for (int i = 0; i < nI; ++i) {
      int k0 = i - bw > 0 ? i - bw : 0;
      double s = y[i];
      for (int k = k0; k < i; ++k) s -= LB(i, k) * y[k];
      y[i] = s / LB(i, i);
    }
    for (int i = nI - 1; i >= 0; --i) {
      int k1 = i + bw < nI - 1 ? i + bw : nI - 1;
      double s = y[i];
      for (int k = i + 1; k <= k1; ++k) s -= LB(k, i) * y[k];
      y[i] = s / LB(i, i);
    }
  }
#undef LB
  free(Lb);
  return 0;
}

/* CSR of A_II with deal.II's row layout: diagonal first, then the other
 * columns ascending, in the unknown numbering given by `perm` (unknown ->
 * row). */
typedef struct csr {
  int n;
  int *rs, *cols, *rdiag;  /* rdiag[i]: first entry right of the diagonal */
  double *val;
} csr;

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return x < y ? -1 : x > y;
}

static void csr_build(const local_sys *L, const int *perm, csr *C) {
  const int nI = L->nI;
  C->n = nI;
  C->rs = malloc(sizeof(int) * (size_t)(nI + 1));
  C->rdiag = malloc(sizeof(int) * (size_t)(nI > 0 ? nI : 1));
  C->cols = malloc(sizeof(int) * (size_t)(nI > 0 ? nI : 1) * L->ns);
  C->val = malloc(sizeof(double) * (size_t)(nI > 0 ? nI : 1) * L->ns);
  int *inv = malloc(sizeof(int) * (size_t)(nI > 0 ? nI : 1));
  for (int u = 0; u < nI; ++u) inv[perm[u]] = u;
  int pos = 0;
  for (int row = 0; row < nI; ++row) {
    int u = inv[row], g = L->node_of[u];
    C->rs[row] = pos;
    int tmp[27][2], cnt = 0;
    double dval = 0.0;
    for (int k = 0; k < L->ns; ++k) {
      int h = nbr(L, g, k);
      if (h < 0) continue;
      int v = L->unk_of[h];
      if (v < 0) continue;
      int col = perm[v];
      if (col == row) { dval = L->st[(size_t)g * L->ns + k]; continue; }
      tmp[cnt][0] = col;
      tmp[cnt][1] = k;
      cnt++;
    }
    C->cols[pos] = row;
    C->val[pos++] = dval;
    qsort(tmp, (size_t)cnt, sizeof(tmp[0]), cmp_int);
    C->rdiag[row] = -1;
    for (int e = 0; e < cnt; ++e) {
      if (C->rdiag[row] < 0 && tmp[e][0] > row) C->rdiag[row] = pos;
      C->cols[pos] = tmp[e][0];
      C->val[pos++] = L->st[(size_t)g * L->ns + tmp[e][1]];
    }
    if (C->rdiag[row] < 0) C->rdiag[row] = pos;
  }
  C->rs[nI] = pos;
  free(inv);
}

static void csr_free(csr *C) {
  free(C->rs); free(C->cols); free(C->rdiag); free(C->val);
}

static void csr_mv(const csr *C, const double *x, double *y) {
  for (int i = 0; i < C->n; ++i) {
    double s = 0.0;
    for (int e = C->rs[i]; e < C->rs[i + 1]; ++e) s += C->val[e] * x[C->cols[e]];
    y[i] = s;
  }
}

/* Standard SSOR preconditioner  P^{-1} = w(2-w) (D + wU)^{-1} D (D + wL)^{-1}
 * (deal.II PreconditionSSOR, relaxation omega): forward sweep over rows in
 * order, scaling by w(2-w) a_ii, backward sweep. */
static void ssor_apply(const csr *C, double om, const double *src, double *dst) {
  const int n = C->n;
  for (int row = 0; row < n; ++row) {
    double s = 0.0;
    for (int e = C->rs[row] + 1; e < C->rdiag[row]; ++e) s += C->val[e] * dst[C->cols[e]];
    dst[row] = (src[row] - s * om) / C->val[C->rs[row]];
  }
  for (int row = 0; row < n; ++row) dst[row] *= om * (2.0 - om) * C->val[C->rs[row]];
  for (int row = n - 1; row >= 0; --row) {
    double s = 0.0;
    for (int e = C->rdiag[row]; e < C->rs[row + 1]; ++e) s += C->val[e] * dst[C->cols[e]];
    dst[row] = (dst[row] - s * om) / C->val[C->rs[row]];
  }
}

static double dot(int n, const double *a, const double *b) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* Preconditioned CG with deal.II SolverCG's control flow
 * (x0 = 0, residual-norm check at step 0 and after every update, failure
 * when the step count reaches maxit).  prec: 1 = SSOR, 2 = Jacobi. */
static int pcg(const csr *C, int prec, double om, const double *b, double *x,
               double tol_abs, int maxit, int *iters) {
  const int n = C->n;
  double *r = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * 3);
  double *z = r + n, *p = z + n, *q = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) { x[i] = 0.0; r[i] = b[i]; }
  double res = sqrt(dot(n, r, r));
  int it = 0, ok = 1;
  if (!(res <= tol_abs)) {
    if (prec == 1) ssor_apply(C, om, r, z);
    else for (int i = 0; i < n; ++i) z[i] = r[i] / C->val[C->rs[i]];
    for (int i = 0; i < n; ++i) p[i] = z[i];
    double rz = dot(n, r, z);
    for (;;) {
      if (it >= maxit) { ok = 0; break; }
      ++it;
      csr_mv(C, p, q);
      double alpha = rz / dot(n, p, q);
      for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
      res = sqrt(dot(n, r, r));
      if (!isfinite(res)) { ok = 0; break; }
      if (res <= tol_abs) break;
      if (prec == 1) ssor_apply(C, om, r, z);
      else for (int i = 0; i < n; ++i) z[i] = r[i] / C->val[C->rs[i]];
      double rz1 = dot(n, r, z);
      double beta = rz1 / rz;
      rz = rz1;
      for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
  }
  *iters = it;
  free(r);
  free(q);
  return ok;
}

/* deal.II numbering of the local dofs: DoFHandler::distribute_dofs visits the
 * active cells in level order -- after refine_global(L) on one coarse cell,
 * the Z-order (Morton) of the N^d lattice with x as the lowest bit -- and
 * numbers each cell's vertices on first touch, in vertex order.  N not a power
 * of two (unreachable with refine_global) falls back to lexicographic cells. */
static void dealii_order(const local_sys *L, int *perm /* unknown -> index */) {
  const int dim = L->dim, N = L->N, n = L->n, nfc = ipow(N, dim);
  int pow2 = (N & (N - 1)) == 0;
  int *num = malloc(sizeof(int) * (size_t)L->nn);
  int *cells = malloc(sizeof(int) * (size_t)nfc);
  for (int g = 0; g < L->nn; ++g) num[g] = -1;
  if (pow2) {
    int bits = 0;
    while ((1 << bits) < N) ++bits;
    for (int m = 0; m < nfc; ++m) {
      int c[MAXD] = {0, 0, 0};
      for (int bt = 0; bt < bits; ++bt)
        for (int a = 0; a < dim; ++a)
          if ((m >> (bt * dim + a)) & 1) c[a] |= 1 << bt;
      cells[m] = c[0] + N * (c[1] + N * c[2]);
    }
  } else {
    for (int m = 0; m < nfc; ++m) cells[m] = m;
  }
  int next = 0;
  for (int m = 0; m < nfc; ++m) {
    int fc = cells[m];
    int cidx[MAXD] = {fc % N, (fc / N) % N, dim == 3 ? fc / (N * N) : 0};
    for (int k = 0; k < (1 << dim); ++k) {
      int ijk[MAXD] = {0, 0, 0};
      for (int a = 0; a < dim; ++a) ijk[a] = cidx[a] + ((k >> a) & 1);
      int g = ijk[0] + n * (ijk[1] + n * ijk[2]);
      if (num[g] < 0) num[g] = next++;
    }
  }
  /* rank the interior unknowns by their global dof number */
  int *key = malloc(sizeof(int) * (size_t)(L->nI > 0 ? L->nI : 1) * 2);
  for (int u = 0; u < L->nI; ++u) { key[2 * u] = num[L->node_of[u]]; key[2 * u + 1] = u; }
  qsort(key, (size_t)L->nI, 2 * sizeof(int), cmp_int);
  for (int r = 0; r < L->nI; ++r) perm[key[2 * r + 1]] = r;
  free(key);
  free(num);
  free(cells);
}

/* One coarse cell: assemble, 2^d Dirichlet solves, epilogue. */
static int run_cell(const oc_batch *b, int32_t cell, double *M, double *F,
                    double *basis, int32_t *iters, double *rel_res) {
  const int dim = b->dim, nv = 1 << dim, N = cell_n(b, cell);
  if (N < 1) return -1;
  const int n = N + 1, nn = ipow(n, dim), ns = ipow(3, dim);
  const double *cr = b->corners + (size_t)cell * nv * dim;
  double *st = malloc(sizeof(double) * (size_t)nn * ns);
  double *bl = malloc(sizeof(double) * (size_t)nn);
  oc_assemble_cell(b, cell, st, bl);
  local_sys L;
  local_sys_init(&L, dim, N, st);
  const int nI = L.nI;
  /* Dirichlet data g_i at every node (used on the boundary only) */
  q1data q;
  q1_setup(b, cell, &q);
  double *phi = malloc(sizeof(double) * (size_t)nv * nn);
  for (int g = 0; g < nn; ++g) {
    int ijk[MAXD] = {g % n, (g / n) % n, dim == 3 ? g / (n * n) : 0};
    double x[MAXD], val[8];
    node_pos(dim, cr, N, ijk, x);
    q1_eval(dim, &q, x, val);
    for (int i = 0; i < nv; ++i) phi[(size_t)i * nn + g] = L.unk_of[g] < 0 ? val[i] : 0.0;
  }
  /* condensed right-hand sides  b_i = -A_IB g_i  (system_rhs = 0 before
   * condense, diffusion_problem_basis.tpp:455-461) */
  double *rhs = malloc(sizeof(double) * (size_t)nv * (nI > 0 ? nI : 1));
  double *tmp = malloc(sizeof(double) * (size_t)nn);
  for (int i = 0; i < nv; ++i) {
    spmv_full(&L, phi + (size_t)i * nn, tmp);
    for (int u = 0; u < nI; ++u) rhs[(size_t)i * nI + u] = -tmp[L.node_of[u]];
  }
  int nfail = 0;
  double *sol = malloc(sizeof(double) * (size_t)nv * (nI > 0 ? nI : 1));
  if (b->solver == OC_SOLVER_DIRECT) {
    memcpy(sol, rhs, sizeof(double) * (size_t)nv * nI);
    if (solve_direct(&L, nv, sol) != 0) nfail = nv;
    if (iters) for (int i = 0; i < nv; ++i) iters[i] = 0;
  } else {
    int *perm = malloc(sizeof(int) * (size_t)(nI > 0 ? nI : 1));
    if (b->solver == OC_SOLVER_SSOR_CG && b->ordering == OC_ORDER_DEALII)
      dealii_order(&L, perm);
    else
      for (int u = 0; u < nI; ++u) perm[u] = u;
    csr C;
    csr_build(&L, perm, &C);
    double *bp = malloc(sizeof(double) * (size_t)(nI > 0 ? nI : 1) * 2), *xp = bp + nI;
    for (int i = 0; i < nv; ++i) {
      for (int u = 0; u < nI; ++u) bp[perm[u]] = rhs[(size_t)i * nI + u];
      double tol = b->tol;
      if (!b->tol_absolute) tol *= sqrt(dot(nI, bp, bp));
      int it = 0;
      int ok = pcg(&C, b->solver == OC_SOLVER_SSOR_CG ? 1 : 2, b->omega, bp, xp,
                   tol, b->maxit, &it);
      if (!ok) nfail++;
      if (iters) iters[i] = it;
      for (int u = 0; u < nI; ++u) sol[(size_t)i * nI + u] = xp[perm[u]];
    }
    free(bp);
    csr_free(&C);
    free(perm);
  }
  /* constraints.distribute: interior values from the solve, boundary = g_i */
  for (int i = 0; i < nv; ++i)
    for (int u = 0; u < nI; ++u) phi[(size_t)i * nn + L.node_of[u]] = sol[(size_t)i * nI + u];
  /* epilogue, diffusion_problem_basis.tpp:245-285:
   *   M(i_test, i_trial) = phi_test . (A phi_trial),  F(i) = phi_i . global_rhs */
  double *Aphi = malloc(sizeof(double) * (size_t)nv * nn);
  for (int j = 0; j < nv; ++j) spmv_full(&L, phi + (size_t)j * nn, Aphi + (size_t)j * nn);
  for (int i = 0; i < nv; ++i) {
    for (int j = 0; j < nv; ++j)
      M[i * nv + j] = dot(nn, phi + (size_t)i * nn, Aphi + (size_t)j * nn);
    F[i] = dot(nn, phi + (size_t)i * nn, bl);
  }
  if (rel_res) {
    for (int i = 0; i < nv; ++i) {
      double rr = 0.0, bb = 0.0;
      for (int u = 0; u < nI; ++u) {
        double r = Aphi[(size_t)i * nn + L.node_of[u]];
        rr += r * r;
        bb += rhs[(size_t)i * nI + u] * rhs[(size_t)i * nI + u];
      }
      rel_res[i] = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
    }
  }
  if (basis) memcpy(basis, phi, sizeof(double) * (size_t)nv * nn);
  free(Aphi); free(sol); free(tmp); free(rhs); free(phi);
  local_sys_free(&L);
  free(st); free(bl);
  return nfail;
}

typedef struct worker_arg {
  const oc_batch *b;
  double *M, *F, *basis, *rel_res;
  int32_t *iters;
  const int64_t *basis_off;
  int next;
  int nfail;
  pthread_mutex_t mu;
} worker_arg;

static void *worker(void *p) {
  worker_arg *w = p;
  const int nv = 1 << w->b->dim;
  for (;;) {
    pthread_mutex_lock(&w->mu);
    int c = w->next++;
    pthread_mutex_unlock(&w->mu);
    if (c >= w->b->n_cells) break;
    int f = run_cell(w->b, c, w->M + (size_t)c * nv * nv, w->F + (size_t)c * nv,
                     w->basis ? w->basis + w->basis_off[c] : NULL,
                     w->iters ? w->iters + (size_t)c * nv : NULL,
                     w->rel_res ? w->rel_res + (size_t)c * nv : NULL);
    if (f) {
      pthread_mutex_lock(&w->mu);
      w->nfail += f > 0 ? f : nv;
      pthread_mutex_unlock(&w->mu);
    }
  }
  return NULL;
}

int oc_run_batch(const oc_batch *b, double *M, double *F, double *basis,
                 int32_t *iters, double *rel_res) {
  if (!b || (b->dim != 2 && b->dim != 3) || b->n_cells < 0 || !M || !F) return -1;
  if (b->coef.kind == OC_COEF_SPHERES) {
    pthread_mutex_lock(&g_sphere_mu);
    if (g_sg_src != b->coef.spheres || g_sg_n != b->coef.n_spheres || g_sg_dim != b->dim)
      sphere_grid_build(b->dim, b->coef.spheres, b->coef.n_spheres);
    pthread_mutex_unlock(&g_sphere_mu);
  }
  const int nv = 1 << b->dim;
  int64_t *off = malloc(sizeof(int64_t) * (size_t)(b->n_cells + 1));
  off[0] = 0;
  for (int c = 0; c < b->n_cells; ++c)
    off[c + 1] = off[c] + (int64_t)nv * ipow(cell_n(b, c) + 1, b->dim);
  worker_arg w = {b, M, F, basis, rel_res, iters, off, 0, 0, PTHREAD_MUTEX_INITIALIZER};
  int nt = b->nthreads > 0 ? b->nthreads : 1;
  if (nt > 256) nt = 256;
  if (nt == 1) {
    worker(&w);
  } else {
    pthread_t th[256];
    for (int t = 0; t < nt; ++t) pthread_create(&th[t], NULL, worker, &w);
    for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
  }
  free(off);
  return w.nfail;
}

/* ------------------------------------------------------------------------ */
/* coarse problem, diffusion_problem_ms.tpp:91-296                           */
/* ------------------------------------------------------------------------ */

void oc_unit_cube_corners(int32_t dim, int32_t K, double *corners) {
  const int nv = 1 << dim, nc = ipow(K, dim);
  for (int c = 0; c < nc; ++c) {
    int cidx[MAXD] = {c % K, (c / K) % K, dim == 3 ? c / (K * K) : 0};
    for (int v = 0; v < nv; ++v)
      for (int a = 0; a < dim; ++a)
        corners[((size_t)c * nv + v) * dim + a] = (double)(cidx[a] + ((v >> a) & 1)) / K;
  }
}

int oc_coarse_solve(int32_t dim, int32_t K, const double *M, const double *F,
                    int32_t bc, double *u) {
  const int nv = 1 << dim, n = K + 1, nn = ipow(n, dim), nc = ipow(K, dim);
  /* coarse stiffness as a (3^d) stencil + load */
  const int ns = ipow(3, dim);
  double *st = calloc((size_t)nn * ns, sizeof(double));
  double *rhs = calloc((size_t)nn, sizeof(double));
  double g[2];
  qgauss2(g);
  for (int c = 0; c < nc; ++c) {
    int cidx[MAXD] = {c % K, (c / K) % K, dim == 3 ? c / (K * K) : 0};
    double Fc[8];
    for (int i = 0; i < nv; ++i) Fc[i] = F[(size_t)c * nv + i];
    if (bc == 0) {
      /* Neumann faces with odd boundary id (x=1, y=1, z=1), QGauss<dim-1>(2),
       * diffusion_problem_ms.tpp:206-235; NeumannBC uses x and y only. */
      for (int a = 0; a < dim; ++a) {
        if (cidx[a] != K - 1) continue;
        int nfq = 1 << (dim - 1);
        for (int fq = 0; fq < nfq; ++fq) {
          double xi[MAXD], x[MAXD];
          int bt = 0;
          for (int e = 0; e < dim; ++e) {
            if (e == a) { xi[e] = 1.0; continue; }
            xi[e] = g[(fq >> bt) & 1];
            bt++;
          }
          for (int e = 0; e < dim; ++e) x[e] = (cidx[e] + xi[e]) / K;
          double gv = cos(2 * OC_PI_D * x[0]) * cos(2 * OC_PI_D * x[1]);
          double JxW = pow(1.0 / K, dim - 1) / nfq;
          for (int i = 0; i < nv; ++i) {
            double psi = 1.0;
            for (int e = 0; e < dim; ++e) psi *= ((i >> e) & 1) ? xi[e] : 1.0 - xi[e];
            Fc[i] += gv * psi * JxW;
          }
        }
      }
    }
    for (int i = 0; i < nv; ++i) {
      int ni[MAXD] = {0, 0, 0};
      for (int a = 0; a < dim; ++a) ni[a] = cidx[a] + ((i >> a) & 1);
      int gi = ni[0] + n * (ni[1] + n * ni[2]);
      for (int j = 0; j < nv; ++j) {
        int off[MAXD];
        for (int a = 0; a < dim; ++a) off[a] = ((j >> a) & 1) - ((i >> a) & 1);
        st[(size_t)gi * ns + stencil_slot(dim, off)] += M[(size_t)c * nv * nv + i * nv + j];
      }
      rhs[gi] += Fc[i];
    }
  }
  /* Dirichlet values */
  double *ud = calloc((size_t)nn, sizeof(double));
  int *fixed = calloc((size_t)nn, sizeof(int));
  for (int gidx = 0; gidx < nn; ++gidx) {
    int ijk[MAXD] = {gidx % n, (gidx / n) % n, dim == 3 ? gidx / (n * n) : 0};
    double x[MAXD];
    for (int a = 0; a < dim; ++a) x[a] = (double)ijk[a] / K;
    int on_even = 0, on_any = 0;
    for (int a = 0; a < dim; ++a) {
      if (ijk[a] == 0) on_even = on_any = 1;
      if (ijk[a] == K) on_any = 1;
    }
    if (bc == 0 && on_even) {
      fixed[gidx] = 1;
      ud[gidx] = (x[0] - 0.5) * (x[0] - 0.5) + (x[1] - 0.5) * (x[1] - 0.5);
    } else if (bc == 1 && on_any) {
      fixed[gidx] = 1;
      ud[gidx] = 0.0;
    }
  }
  /* reduced system A_FF u_F = F_F - A_FD u_D via the local_sys machinery */
  int *unk = malloc(sizeof(int) * (size_t)nn), *node = malloc(sizeof(int) * (size_t)nn), nF = 0;
  for (int gidx = 0; gidx < nn; ++gidx) {
    unk[gidx] = fixed[gidx] ? -1 : nF;
    if (!fixed[gidx]) node[nF++] = gidx;
  }
  local_sys L;
  L.dim = dim; L.N = K; L.n = n; L.nn = nn; L.ns = ns; L.nI = nF;
  L.node_of = node; L.unk_of = unk; L.st = st;
  double *y = malloc(sizeof(double) * (size_t)nn);
  spmv_full(&L, ud, y);
  double *sol = malloc(sizeof(double) * (size_t)(nF > 0 ? nF : 1));
  for (int f = 0; f < nF; ++f) sol[f] = rhs[node[f]] - y[node[f]];
  /* banded solve: bandwidth in lexicographic order of free nodes */
  int bwmax = 0;
  for (int f = 0; f < nF; ++f)
    for (int k = 0; k < ns; ++k) {
      int h = nbr(&L, node[f], k);
      if (h >= 0 && unk[h] >= 0 && f - unk[h] > bwmax) bwmax = f - unk[h];
    }
  const int bw = bwmax;
  double *Lb = calloc((size_t)(nF > 0 ? nF : 1) * (bw + 1), sizeof(double));
  int rc = 0;
#define LB(i, j) Lb[(size_t)(i) * (bw + 1) + ((i) - (j))]
  for (int f = 0; f < nF; ++f)
    for (int k = 0; k < ns; ++k) {
      int h = nbr(&L, node[f], k);
      if (h < 0 || unk[h] < 0 || unk[h] > f) continue;
      LB(f, unk[h]) = st[(size_t)node[f] * ns + k];
    }
  for (int j = 0; j < nF && rc == 0; ++j) {
    int k0 = j - bw > 0 ? j - bw : 0;
    double s = LB(j, j);
    for (int k = k0; k < j; ++k) s -= LB(j, k) * LB(j, k);
    if (!(s > 0)) { rc = -2; break; }
    double d = sqrt(s);
    LB(j, j) = d;
    int i1 = j + bw < nF - 1 ? j + bw : nF - 1;
    for (int i = j + 1; i <= i1; ++i) {
      int kk = i - bw > 0 ? i - bw : 0;
      double t = LB(i, j);
      for (int k = kk; k < j; ++k) t -= LB(i, k) * LB(j, k);
      LB(i, j) = t / d;
    }
  }
  if (rc == 0) {
    for (int i = 0; i < nF; ++i) {
      int k0 = i - bw > 0 ? i - bw : 0;
      double s = sol[i];
      for (int k = k0; k < i; ++k) s -= LB(i, k) * sol[k];
      sol[i] = s / LB(i, i);
    }
    for (int i = nF - 1; i >= 0; --i) {
      int k1 = i + bw < nF - 1 ? i + bw : nF - 1;
      double s = sol[i];
      for (int k = i + 1; k <= k1; ++k) s -= LB(k, i) * sol[k];
      sol[i] = s / LB(i, i);
    }
    for (int gidx = 0; gidx < nn; ++gidx) u[gidx] = fixed[gidx] ? ud[gidx] : sol[unk[gidx]];
  }
#undef LB
  free(Lb); free(sol); free(y); free(unk); free(node); free(ud); free(fixed);
  free(st); free(rhs);
  return rc;
}
