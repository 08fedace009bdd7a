// msfem_gpu.cu -- libmsfem_gpu.so: C-ABI (include/msfem_gpu.h) over the
// sm_103a multiscale-basis kernels.
//
// Replaces, per batch of coarse cells, DiffusionProblemBasis<dim>::run()
// (include/base/diffusion_problem_basis.tpp:438-474) as called by
// DiffusionProblemMultiscale<dim>::initialize_and_compute_basis
// (include/base/diffusion_problem_ms.tpp:81-87).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "msfem_common.cuh"
#include "msfem_cnn.cuh"
#include "msfem_gpu.h"
#include "msfem_launch.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

#define MSFEM_CUDA(call)                                                        \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess)                                                      \
      return fail(MSFEM_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

struct DevBuf {
  void *ptr = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

// Autotuned launch choice for one (dim, N class, precision).
struct Tune {
  int variant = 0;
  int check_interval = 0;
  float inner_tol = 1e-6f;
  float cheb_ratio = 30.0f;
  double ms_per_solve = 0.0;
};

}  // namespace

struct msfem_handle {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // second stream of the size-class split (3D mixed, slab-cluster shape):
  // the small cells run there beside the cluster launch, joined by events
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // inputs staged from the host / internal scratch
  DevBuf corners, nfine, order, queue, qp, qpoff, warm, boff, modes, spheres, sgrid_start, sgrid_ids;
  DevBuf fqp, fqpoff;  // right-hand side tabulated at the Gauss points
  // outputs staged to the host / internal
  DevBuf M, F, basis, status, iters, relres, refine;
  DevBuf work;  // per-CTA workspace slots of the 3D kernels
  // learned warm start
  msfem_surrogate *surrogate = nullptr;
  DevBuf feat, delta, warm_pred;
  // CUDA graph of the last device-resident launch sequence
  bool use_graphs = true;
  std::string graph_key;
  cudaGraphExec_t graph_exec = nullptr;
  int64_t graph_launches = 0;
  int64_t graph_captures = 0;
  // autotuned launch choices, keyed by (dim, N class, precision)
  std::map<int, Tune> tuning;
};

namespace msfem {

// ---------------------------------------------------------------------------
// Coefficient tabulation at the QGauss(2) points (analytic kinds), layout
// [comp][q][fine cell] per cell.  One CTA per coarse cell.
// ---------------------------------------------------------------------------
struct TabParams {
  int dim, n_cells, n_fine_uniform, kind, ncomp, n_modes;
  const double *corners;
  const int32_t *n_fine;
  const int64_t *offset;
  double cparams[8];
  const double *modes;      // [fields][n_modes][5]
  const double *spheres;    // [n][4]
  const int32_t *sg_start;  // sphere hash grid
  const int32_t *sg_ids;
  int sg_G;
  double sg_h;
  double *out;
};

__device__ double fourier_field(const TabParams &t, int f, const double *x) {
  double g = 0.0;
  const double *md = t.modes + (int64_t)f * t.n_modes * 5;
  for (int m = 0; m < t.n_modes; ++m) {
    const double ph = md[5 * m] * x[0] + md[5 * m + 1] * x[1] +
                      (t.dim == 3 ? md[5 * m + 2] * x[2] : 0.0) + md[5 * m + 4];
    g = fma(md[5 * m + 3], cos(ph), g);
  }
  return g;
}

__device__ bool inside_sphere(const TabParams &t, const double *x) {
  int idx[3] = {0, 0, 0};
  for (int a = 0; a < t.dim; ++a) {
    int i = (int)floor(x[a] / t.sg_h);
    idx[a] = min(max(i, 0), t.sg_G - 1);
  }
  const int g = idx[0] + t.sg_G * (idx[1] + (t.dim == 3 ? t.sg_G * idx[2] : 0));
  for (int e = t.sg_start[g]; e < t.sg_start[g + 1]; ++e) {
    const double *s = t.spheres + 4 * t.sg_ids[e];
    double d2 = 0.0;
    for (int a = 0; a < t.dim; ++a) d2 += (x[a] - s[a]) * (x[a] - s[a]);
    if (d2 <= s[3] * s[3]) return true;
  }
  return false;
}

// Random-Fourier fields on an affine cell.  Along a lattice row of Gauss
// points (fixed y[, z] and Gauss-point offsets, x advancing by one fine cell)
// the point moves by the constant vector e1 = (v1 - v0) / N, so every mode's
// phase advances by the constant k . e1: cos and sin of the phase follow the
// angle-addition recurrence (one 2 x 2 rotation per point) instead of one cos
// per point and mode.  Each segment of kSeg points starts from a direct
// sincos of its first phase, which bounds the recurrence's rounding drift to
// kSeg steps (a few 1e-15 relative).  Pass 1: one task per (field, row,
// segment) sums its field along the segment into the output block (as
// scratch, component f = field f).  Pass 2 (2D): each point's three fields
// become the tensor components in place.
constexpr int kSeg = 16;

__device__ void tabulate_fourier_affine(const TabParams &t, const double *cr, int N, int nfc, double *out,
                                        double *rot /* [fields][n_modes][2] shared */) {
  const int dim = t.dim, nv = 1 << dim;
  const int nf = dim == 2 ? 3 : 1;
  const double invN = 1.0 / N;
  double e[3][3];  // e[a] = (v_{2^a} - v0) / N
  for (int a = 0; a < dim; ++a)
    for (int b = 0; b < dim; ++b) e[a][b] = (cr[(1 << a) * dim + b] - cr[b]) * invN;
  // cos / sin of each mode's phase step along x
  for (int i = threadIdx.x; i < nf * t.n_modes; i += blockDim.x) {
    const double *md = t.modes + (int64_t)i * 5;
    const double dph = md[0] * e[0][0] + md[1] * e[0][1] + (dim == 3 ? md[2] * e[0][2] : 0.0);
    sincos(dph, &rot[2 * i + 1], &rot[2 * i]);
  }
  __syncthreads();
  const int nseg = (N + kSeg - 1) / kSeg;
  const int rows = (dim == 2 ? N : N * N) * nv;  // (y[, z], Gauss-point offsets)
  const int tasks = nf * rows * nseg;
  for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
    const int seg = task % nseg, row = (task / nseg) % rows, f = task / (nseg * rows);
    const int q = row % nv, yz = row / nv;
    const int cy = yz % N, cz = dim == 3 ? yz / N : 0;
    const int cx0 = seg * kSeg;
    const double u[3] = {cx0 + gauss2(q & 1), cy + gauss2((q >> 1) & 1), cz + gauss2((q >> 2) & 1)};
    double x0[3];
    for (int b = 0; b < dim; ++b) {
      x0[b] = cr[b];
      for (int a = 0; a < dim; ++a) x0[b] = fma(e[a][b], u[a], x0[b]);
    }
    double g[kSeg];
#pragma unroll
    for (int j = 0; j < kSeg; ++j) g[j] = 0.0;
    const double *md = t.modes + (int64_t)f * t.n_modes * 5;
    const double *rf = rot + 2 * f * t.n_modes;
    for (int m = 0; m < t.n_modes; ++m) {
      const double ph = md[5 * m] * x0[0] + md[5 * m + 1] * x0[1] + (dim == 3 ? md[5 * m + 2] * x0[2] : 0.0) +
                        md[5 * m + 4];
      double c, sn;
      sincos(ph, &sn, &c);
      const double amp = md[5 * m + 3], cd = rf[2 * m], sd = rf[2 * m + 1];
#pragma unroll
      for (int j = 0; j < kSeg; ++j) {
        g[j] = fma(amp, c, g[j]);
        const double c2 = c * cd - sn * sd;
        sn = fma(sn, cd, c * sd);
        c = c2;
      }
    }
    const int fc0 = (cz * N + cy) * N + cx0;
    const int cnt = min(kSeg, N - cx0);
    if (dim == 2) {
      double *o = out + ((int64_t)f * nv + q) * nfc + fc0;
#pragma unroll
      for (int j = 0; j < kSeg; ++j)
        if (j < cnt) o[j] = g[j];
    } else {
      // 3D: a = exp(g1); ncomp 6 writes the diagonal tensor a I
#pragma unroll
      for (int j = 0; j < kSeg; ++j)
        if (j < cnt) {
          const double a = exp(g[j]);
          if (t.ncomp == 1) {
            out[(int64_t)q * nfc + fc0 + j] = a;
          } else {
            const double comp[6] = {a, 0.0, 0.0, a, 0.0, a};
            for (int k = 0; k < 6; ++k) out[((int64_t)k * nv + q) * nfc + fc0 + j] = comp[k];
          }
        }
    }
  }
  if (dim == 3) return;
  __syncthreads();
  // 2D: A = R(theta) diag(e^g1, e^g2) R(theta)^T from the three fields, in place
  for (int i = threadIdx.x; i < nv * nfc; i += blockDim.x) {
    const double g1 = out[i], g2 = out[(int64_t)nv * nfc + i], th = out[2 * (int64_t)nv * nfc + i];
    double sn, cn;
    sincos(th, &sn, &cn);
    const double e1 = exp(g1), e2 = exp(g2);
    out[i] = cn * cn * e1 + sn * sn * e2;
    out[(int64_t)nv * nfc + i] = cn * sn * (e1 - e2);
    out[2 * (int64_t)nv * nfc + i] = sn * sn * e1 + cn * cn * e2;
  }
}

__device__ __forceinline__ bool affine_corners(const double *cr, int dim) {
  for (int k = 0; k < (1 << dim); ++k)
    for (int a = 0; a < dim; ++a) {
      const double pred = cr[a] + ((k & 1) ? cr[dim + a] - cr[a] : 0.0) +
                          ((k & 2) ? cr[2 * dim + a] - cr[a] : 0.0) + ((k & 4) ? cr[4 * dim + a] - cr[a] : 0.0);
      if (pred != cr[k * dim + a]) return false;
    }
  return true;
}

__global__ void tabulate_kernel(const TabParams t) {
  extern __shared__ double tab_rot[];
  const int cell = blockIdx.x;
  if (cell >= t.n_cells) return;
  const int dim = t.dim, nv = 1 << dim;
  const int N = t.n_fine ? t.n_fine[cell] : t.n_fine_uniform;
  int nfc = N * N;
  if (dim == 3) nfc *= N;
  const double *cr = t.corners + (int64_t)cell * nv * dim;
  double *out = t.out + (t.offset ? t.offset[cell] : (int64_t)cell * t.ncomp * nv * nfc);
  if (t.kind == MSFEM_COEF_FOURIER && (dim == 3 || t.ncomp == 3) && affine_corners(cr, dim)) {
    tabulate_fourier_affine(t, cr, N, nfc, out, tab_rot);
    return;
  }
  const double invN = 1.0 / N;
  for (int fc = threadIdx.x; fc < nfc; fc += blockDim.x) {
    const int cx = fc % N, cy = (fc / N) % N, cz = dim == 3 ? fc / (N * N) : 0;
    for (int q = 0; q < nv; ++q) {
      double tt[3];
      tt[0] = (cx + gauss2(q & 1)) * invN;
      tt[1] = (cy + gauss2((q >> 1) & 1)) * invN;
      tt[2] = (cz + gauss2((q >> 2) & 1)) * invN;
      double x[3] = {0.0, 0.0, 0.0};
      for (int v = 0; v < nv; ++v) {
        double w = 1.0;
        for (int a = 0; a < dim; ++a) w *= ((v >> a) & 1) ? tt[a] : 1.0 - tt[a];
        for (int a = 0; a < dim; ++a) x[a] += w * cr[v * dim + a];
      }
      double comp[6] = {0, 0, 0, 0, 0, 0};
      double a_scalar = 0.0;
      bool scalar = true;
      switch (t.kind) {
      case MSFEM_COEF_REFERENCE: {
        const double c = 1.0 * (1.0 - 0.9999 * (0.5 * sin(2 * kPiD * 57 * x[0]) +
                                                0.5 * sin(2 * kPiD * 57 * x[1])));
        for (int k = 0; k < (dim == 2 ? 3 : 6); ++k) comp[k] = c * t.cparams[k];
        scalar = false;
        break;
      }
      case MSFEM_COEF_SINSIN: {
        const double ie = 2.0 / t.cparams[1];
        double s = sinpi(x[0] * ie) * sinpi(x[1] * ie);
        if (dim == 3) s *= sinpi(x[2] * ie);
        a_scalar = 1.0 + t.cparams[0] * s;
        break;
      }
      case MSFEM_COEF_FOURIER: {
        if (dim == 2) {
          const double g1 = fourier_field(t, 0, x), g2 = fourier_field(t, 1, x);
          const double th = fourier_field(t, 2, x);
          double sn, cn;
          sincos(th, &sn, &cn);
          const double e1 = exp(g1), e2 = exp(g2);
          // R diag(e1,e2) R^T, R = [[c,-s],[s,c]]
          comp[0] = cn * cn * e1 + sn * sn * e2;
          comp[1] = cn * sn * (e1 - e2);
          comp[2] = sn * sn * e1 + cn * cn * e2;
          scalar = false;
        } else {
          a_scalar = exp(fourier_field(t, 0, x));
        }
        break;
      }
      case MSFEM_COEF_SPHERES:
        a_scalar = inside_sphere(t, x) ? t.cparams[0] : 1.0;
        break;
      default:  // CONSTANT
        for (int k = 0; k < (dim == 2 ? 3 : 6); ++k) comp[k] = t.cparams[k];
        scalar = false;
        break;
      }
      if (scalar) {
        if (t.ncomp == 1) {
          comp[0] = a_scalar;
        } else if (dim == 2) {
          comp[0] = a_scalar; comp[1] = 0.0; comp[2] = a_scalar;
        } else {
          comp[0] = a_scalar; comp[1] = comp[2] = 0.0; comp[3] = a_scalar; comp[4] = 0.0; comp[5] = a_scalar;
        }
      }
      // ncomp == 1 with a tensor kind keeps a11 (caller's choice)
      for (int k = 0; k < t.ncomp; ++k) out[((int64_t)k * nv + q) * nfc + fc] = comp[k];
    }
  }
}

}  // namespace msfem

namespace {

using msfem::KernelParams;

int ipow(int a, int e) {
  int r = 1;
  while (e-- > 0) r *= a;
  return r;
}

int cell_N(const msfem_batch_desc *d, const std::vector<int32_t> &nf, int c) {
  return d->n_fine_per_cell ? nf[c] : d->n_fine;
}

// Reference MatrixCoeff rotation products R R^T (matrix_coeff.tpp:17-41).
void reference_rrt(int dim, double *out) {
  const double pi_d = msfem::kPiD;
  const double al = pi_d / 3, be = pi_d / 6, ga = pi_d / 4;
  double R[9];
  if (dim == 2) {
    R[0] = cos(al); R[1] = sin(al); R[2] = -sin(al); R[3] = cos(al);
    out[0] = R[0] * R[0] + R[1] * R[1];
    out[1] = R[0] * R[2] + R[1] * R[3];
    out[2] = R[2] * R[2] + R[3] * R[3];
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
    auto rr = [&](int i, int j) {
      return R[3 * i] * R[3 * j] + R[3 * i + 1] * R[3 * j + 1] + R[3 * i + 2] * R[3 * j + 2];
    };
    out[0] = rr(0, 0); out[1] = rr(0, 1); out[2] = rr(0, 2);
    out[3] = rr(1, 1); out[4] = rr(1, 2); out[5] = rr(2, 2);
  }
}

template <typename T>
int upload(msfem_handle *h, DevBuf &buf, const T *src, size_t count, bool device,
           const T **dst, int64_t *h2d) {
  if (count == 0) {
    *dst = nullptr;
    return MSFEM_OK;
  }
  if (device) {
    *dst = src;
    return MSFEM_OK;
  }
  // Large inputs in pinned (page-locked, device-mapped) host memory are read
  // in place by the kernels over the CPU-GPU link (NVLink-C2C on Grace
  // nodes): each value is read once, spread over the whole launch, instead
  // of a copy that must finish before the launch starts.  The caller's buffer
  // is only read while the call runs (host-memory calls synchronise before
  // returning).  Pageable memory is copied.
  if (count * sizeof(T) >= (size_t(1) << 20)) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, src) == cudaSuccess && a.type == cudaMemoryTypeHost &&
        a.devicePointer != nullptr) {
      *dst = static_cast<const T *>(a.devicePointer);
      *h2d += (int64_t)(count * sizeof(T));
      return MSFEM_OK;
    }
    (void)cudaGetLastError();
  }
  MSFEM_CUDA(buf.ensure(count * sizeof(T)));
  MSFEM_CUDA(cudaMemcpyAsync(buf.ptr, src, count * sizeof(T), cudaMemcpyHostToDevice, h->stream));
  *h2d += (int64_t)(count * sizeof(T));
  *dst = buf.as<T>();
  return MSFEM_OK;
}

using msfem::Launch;

// Compiled launch shapes per (dim, N class, precision); index 0 is the default.
std::vector<Launch> candidates(int dim, int nmax, bool mixed) {
  if (dim == 2) return nmax <= MSFEM_MAX_N_2D ? msfem::candidates_2d(nmax, mixed) : std::vector<Launch>{};
  if (nmax > MSFEM_MAX_N_3D) return {};
  return mixed ? msfem::candidates_3d_mixed() : msfem::candidates_3d_fp64();
}

int size_class(int dim, int nmax) {
  if (dim == 2) return nmax <= 16 ? 16 : 32;
  return nmax <= 8 ? 8 : (nmax <= 16 ? 16 : 24);
}

int tune_key(int dim, int nmax, bool mixed) {
  return dim * 1000 + size_class(dim, nmax) * 10 + (mixed ? 1 : 0);
}

// Sphere hash grid (uniform cells of width >= 2 r_max; each sphere listed in
// every grid cell its bounding box touches).
void build_sphere_grid(int dim, const double *sp, int n, std::vector<int32_t> &start,
                       std::vector<int32_t> &ids, int *Gout, double *hout) {
  double rmax = 0.0;
  for (int s = 0; s < n; ++s) rmax = std::max(rmax, sp[4 * s + 3]);
  double h = std::max(2.0 * rmax, 1e-3);
  int G = std::min(256, std::max(1, (int)std::ceil(1.0 / h)));
  h = 1.0 / G;
  const int ncell = ipow(G, dim);
  std::vector<int32_t> cnt(ncell + 1, 0);
  for (int pass = 0; pass < 2; ++pass) {
    for (int s = 0; s < n; ++s) {
      int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
      for (int a = 0; a < dim; ++a) {
        const double c = sp[4 * s + a], r = sp[4 * s + 3];
        lo[a] = std::max(0, (int)std::floor((c - r) / h));
        hi[a] = std::min(G - 1, (int)std::floor((c + r) / h));
      }
      for (int k = lo[2]; k <= hi[2]; ++k)
        for (int j = lo[1]; j <= hi[1]; ++j)
          for (int i = lo[0]; i <= hi[0]; ++i) {
            const int g = i + G * (j + (dim == 3 ? G * k : 0));
            if (pass == 0) cnt[g + 1]++;
            else ids[cnt[g]++] = s;
          }
    }
    if (pass == 0) {
      for (int g = 0; g < ncell; ++g) cnt[g + 1] += cnt[g];
      start = cnt;
      ids.assign(std::max<int32_t>(1, cnt[ncell]), 0);
    }
  }
  *Gout = G;
  *hout = h;
}

int validate(const msfem_batch_desc *d) {
  if (!d) return fail(MSFEM_ERR_INVALID_ARG, "descriptor is NULL");
  if (d->dim != 2 && d->dim != 3) return fail(MSFEM_ERR_INVALID_ARG, "dim must be 2 or 3");
  if (d->n_cells < 0) return fail(MSFEM_ERR_INVALID_ARG, "n_cells < 0");
  if (d->n_cells > 0 && !d->corners) return fail(MSFEM_ERR_INVALID_ARG, "corners is NULL");
  if (!d->n_fine_per_cell) {
    const int nmax = d->dim == 2 ? MSFEM_MAX_N_2D : MSFEM_MAX_N_3D;
    if (d->n_fine < 1 || d->n_fine > nmax)
      return fail(MSFEM_ERR_INVALID_ARG, "n_fine out of range [1, " + std::to_string(nmax) + "]");
  }
  if (d->precision != MSFEM_PREC_FP64 && d->precision != MSFEM_PREC_MIXED)
    return fail(MSFEM_ERR_INVALID_ARG, "unknown precision");
  if (d->memory != MSFEM_MEM_HOST && d->memory != MSFEM_MEM_DEVICE)
    return fail(MSFEM_ERR_INVALID_ARG, "unknown memory kind");
  if (!(d->tol > 0.0) || !std::isfinite(d->tol)) return fail(MSFEM_ERR_INVALID_ARG, "tol must be > 0");
  if (d->maxit < 1) return fail(MSFEM_ERR_INVALID_ARG, "maxit must be >= 1");
  if (d->check_interval < 0) return fail(MSFEM_ERR_INVALID_ARG, "check_interval < 0");
  if (d->warm_start != MSFEM_WARM_NONE && d->warm_start != MSFEM_WARM_USER &&
      d->warm_start != MSFEM_WARM_SURROGATE)
    return fail(MSFEM_ERR_INVALID_ARG, "unknown warm_start");
  if (d->warm_start == MSFEM_WARM_USER && d->n_cells > 0 && !d->warm_basis)
    return fail(MSFEM_ERR_INVALID_ARG, "warm_basis is NULL");
  if (d->tol_absolute != 0 && d->tol_absolute != 1) return fail(MSFEM_ERR_INVALID_ARG, "tol_absolute must be 0 or 1");
  if (d->reserved0 != 0) return fail(MSFEM_ERR_INVALID_ARG, "reserved0 must be 0");
  if (d->f_qp_offset && !d->f_qp_values)
    return fail(MSFEM_ERR_INVALID_ARG, "f_qp_offset given without f_qp_values");
  const msfem_coef_desc &c = d->coef;
  switch (c.kind) {
  case MSFEM_COEF_CONSTANT:
  case MSFEM_COEF_REFERENCE:
  case MSFEM_COEF_SINSIN:
    break;
  case MSFEM_COEF_FOURIER:
    if (!c.modes || c.n_modes < 1) return fail(MSFEM_ERR_INVALID_ARG, "FOURIER needs modes");
    break;
  case MSFEM_COEF_SPHERES:
    if (c.n_spheres < 0 || (c.n_spheres > 0 && !c.spheres))
      return fail(MSFEM_ERR_INVALID_ARG, "SPHERES needs spheres");
    break;
  case MSFEM_COEF_TABULATED: {
    const int full = d->dim == 2 ? 3 : 6;
    if (c.ncomp != 1 && c.ncomp != full)
      return fail(MSFEM_ERR_INVALID_ARG, "TABULATED ncomp must be 1 or d(d+1)/2");
    if (d->n_cells > 0 && !c.qp_values) return fail(MSFEM_ERR_INVALID_ARG, "qp_values is NULL");
    break;
  }
  default:
    return fail(MSFEM_ERR_INVALID_ARG, "unknown coefficient kind");
  }
  if (c.kind == MSFEM_COEF_SINSIN && !(c.params[1] != 0.0))
    return fail(MSFEM_ERR_INVALID_ARG, "SINSIN eps must be nonzero");
  return MSFEM_OK;
}

// Fill the per-cell N vector on the host (copying it from the device when needed).
int host_nfine(msfem_handle *h, const msfem_batch_desc *d, std::vector<int32_t> &nf) {
  nf.clear();
  if (!d->n_fine_per_cell) return MSFEM_OK;
  nf.resize(d->n_cells);
  if (d->memory == MSFEM_MEM_DEVICE) {
    MSFEM_CUDA(cudaMemcpyAsync(nf.data(), d->n_fine_per_cell, sizeof(int32_t) * d->n_cells,
                               cudaMemcpyDeviceToHost, h->stream));
    MSFEM_CUDA(cudaStreamSynchronize(h->stream));
  } else {
    std::memcpy(nf.data(), d->n_fine_per_cell, sizeof(int32_t) * d->n_cells);
  }
  const int nmax = d->dim == 2 ? MSFEM_MAX_N_2D : MSFEM_MAX_N_3D;
  for (int c = 0; c < d->n_cells; ++c)
    if (nf[c] < 1 || nf[c] > nmax)
      return fail(MSFEM_ERR_INVALID_ARG, "n_fine_per_cell[" + std::to_string(c) + "] out of range");
  return MSFEM_OK;
}

// Evaluate an analytic coefficient into a device TABULATED buffer.
int run_tabulate(msfem_handle *h, const msfem_batch_desc *d, const std::vector<int32_t> &nf,
                 const double *corners_dev, const int32_t *nfine_dev, int ncomp, double *out_dev,
                 const int64_t *offsets_dev, int64_t *h2d, int *launches) {
  msfem::TabParams t{};
  t.dim = d->dim;
  t.n_cells = d->n_cells;
  t.n_fine_uniform = d->n_fine;
  t.kind = d->coef.kind;
  t.ncomp = ncomp;
  t.corners = corners_dev;
  t.n_fine = nfine_dev;
  t.offset = offsets_dev;
  t.out = out_dev;
  for (int k = 0; k < 8; ++k) t.cparams[k] = d->coef.params[k];
  if (t.kind == MSFEM_COEF_REFERENCE) reference_rrt(d->dim, t.cparams);
  const bool dev = d->memory == MSFEM_MEM_DEVICE;
  if (t.kind == MSFEM_COEF_FOURIER) {
    const int nf_fields = d->dim == 2 ? 3 : 1;
    const double *m = nullptr;
    int rc = upload<double>(h, h->modes, d->coef.modes, (size_t)nf_fields * d->coef.n_modes * 5, dev, &m, h2d);
    if (rc) return rc;
    t.modes = m;
    t.n_modes = d->coef.n_modes;
  }
  if (t.kind == MSFEM_COEF_SPHERES) {
    std::vector<int32_t> start, ids;
    int G = 1;
    double hh = 1.0;
    build_sphere_grid(d->dim, d->coef.spheres, d->coef.n_spheres, start, ids, &G, &hh);
    const double *sp = nullptr;
    const int32_t *st = nullptr, *id = nullptr;
    int rc = upload<double>(h, h->spheres, d->coef.spheres, (size_t)std::max(1, d->coef.n_spheres) * 4,
                            false, &sp, h2d);
    if (rc) return rc;
    rc = upload<int32_t>(h, h->sgrid_start, start.data(), start.size(), false, &st, h2d);
    if (rc) return rc;
    rc = upload<int32_t>(h, h->sgrid_ids, ids.data(), ids.size(), false, &id, h2d);
    if (rc) return rc;
    t.spheres = sp;
    t.sg_start = st;
    t.sg_ids = id;
    t.sg_G = G;
    t.sg_h = hh;
  }
  if (d->n_cells == 0) return MSFEM_OK;
  // shared memory: the per-mode phase-step rotations of the FOURIER kind
  const size_t rot_bytes =
      t.kind == MSFEM_COEF_FOURIER ? sizeof(double) * 2 * (d->dim == 2 ? 3 : 1) * (size_t)t.n_modes : 0;
  if (rot_bytes > 48 * 1024)
    MSFEM_CUDA(cudaFuncSetAttribute(msfem::tabulate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)rot_bytes));
  msfem::tabulate_kernel<<<d->n_cells, 256, rot_bytes, h->stream>>>(t);
  MSFEM_CUDA(cudaGetLastError());
  (*launches)++;
  (void)nf;
  return MSFEM_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Scratch of msfem_run_batch_noalloc: one fixed device array per GPU that
// loads this library (held until the process exits).  Layout: work-queue
// counter in the first 256 bytes, then rel_res [MAX] doubles, then
// refinements [MAX] int32.  Device code could name it directly; host code
// must fetch its device address with cudaGetSymbolAddress (the host-side name
// is only a stand-in for the device object).
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoallocRelres = 256;
constexpr size_t kNoallocRefine = kNoallocRelres + sizeof(double) * MSFEM_NOALLOC_MAX_CELLS;
constexpr size_t kNoallocBytes = kNoallocRefine + sizeof(int32_t) * MSFEM_NOALLOC_MAX_CELLS;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {};

// Once per device, with that device current: the scratch array's address.
int noalloc_scratch(int device, void **out) {
  if (device < 0 || device >= kMaxDevices) return fail(MSFEM_ERR_INVALID_ARG, "device id out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(MSFEM_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_noalloc_ptr[device] = ptr;
  }
  *out = g_noalloc_ptr[device];
  return MSFEM_OK;
}

}  // namespace

extern "C" {

int msfem_run_batch_noalloc(const msfem_batch_desc *d, double *M, double *F, double *basis,
                            int32_t *cell_status, int32_t *iterations, void *stream) {
  int rc = validate(d);
  if (rc) return rc;
  if (d->dim != 2) return fail(MSFEM_ERR_UNSUPPORTED, "msfem_run_batch_noalloc: 2D only");
  if (d->memory != MSFEM_MEM_DEVICE)
    return fail(MSFEM_ERR_INVALID_ARG, "msfem_run_batch_noalloc: desc->memory must be MSFEM_MEM_DEVICE");
  if (d->n_fine_per_cell)
    return fail(MSFEM_ERR_INVALID_ARG, "msfem_run_batch_noalloc: uniform N only (n_fine_per_cell must be NULL)");
  if (d->n_cells > MSFEM_NOALLOC_MAX_CELLS)
    return fail(MSFEM_ERR_INVALID_ARG, "msfem_run_batch_noalloc: n_cells " + std::to_string(d->n_cells) +
                                           " exceeds MSFEM_NOALLOC_MAX_CELLS (" +
                                           std::to_string(MSFEM_NOALLOC_MAX_CELLS) + ")");
  const int kind = d->coef.kind;
  if (kind != MSFEM_COEF_CONSTANT && kind != MSFEM_COEF_REFERENCE && kind != MSFEM_COEF_SINSIN &&
      kind != MSFEM_COEF_TABULATED)
    return fail(MSFEM_ERR_UNSUPPORTED, "msfem_run_batch_noalloc: tabulate FOURIER/SPHERES coefficients first");
  if (d->warm_start == MSFEM_WARM_SURROGATE)
    return fail(MSFEM_ERR_UNSUPPORTED,
                "msfem_run_batch_noalloc: MSFEM_WARM_SURROGATE needs a handle and its buffers; use msfem_run_batch");
  if (d->n_cells > 0 && (!M || !F || !cell_status))
    return fail(MSFEM_ERR_INVALID_ARG, "msfem_run_batch_noalloc: M, F and cell_status are required");
  if (d->n_cells == 0) return MSFEM_OK;
  const bool mixed = d->precision == MSFEM_PREC_MIXED;
  const std::vector<Launch> cands = candidates(2, d->n_fine, mixed);
  if (cands.empty()) return fail(MSFEM_ERR_UNSUPPORTED, "no kernel for this N");
  // the default compiled shape and parameters: this entry has no handle, so
  // no autotuned choice applies
  const Launch L = cands[0];
  int device = 0;
  MSFEM_CUDA(cudaGetDevice(&device));
  void *scratch = nullptr;
  if ((rc = noalloc_scratch(device, &scratch))) return rc;
  unsigned char *base = static_cast<unsigned char *>(scratch);

  KernelParams p{};
  p.dim = 2;
  p.n_cells = d->n_cells;
  p.n_fine_uniform = d->n_fine;
  p.corners = d->corners;
  p.n_fine = nullptr;
  p.order = nullptr;
  p.queue = reinterpret_cast<unsigned int *>(base);
  p.coef_kind = kind;
  p.ncomp = d->coef.ncomp;
  for (int k = 0; k < 8; ++k) p.cparams[k] = d->coef.params[k];
  if (kind == MSFEM_COEF_REFERENCE) reference_rrt(2, p.cparams);
  p.qp_values = d->coef.qp_values;
  p.qp_offset = d->coef.qp_offset;
  p.f_value = d->f_value;
  p.f_qp = d->f_qp_values;
  p.f_qp_offset = d->f_qp_offset;
  p.tol = d->tol;
  p.tol_abs = d->tol_absolute;
  p.maxit = d->maxit;
  p.check_interval = d->check_interval;
  p.inner_tol = Tune().inner_tol;
  p.inner_maxit = std::max(1, std::min(d->maxit, 1000));
  p.max_refine = 40;
  p.cheb_ratio = Tune().cheb_ratio;
  p.warm_basis = d->warm_start == MSFEM_WARM_USER ? d->warm_basis : nullptr;
  p.basis_offset = nullptr;
  p.M = M;
  p.F = F;
  p.basis = basis;
  p.status = cell_status;
  p.iters = iterations;
  p.rel_res = reinterpret_cast<double *>(base + kNoallocRelres);
  p.refinements = reinterpret_cast<int32_t *>(base + kNoallocRefine);

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  MSFEM_CUDA(cudaFuncSetAttribute(L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
  int per_sm = 0, sms = 0;
  MSFEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, L.fn, L.nt, L.smem));
  MSFEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  if (per_sm < 1) return fail(MSFEM_ERR_UNSUPPORTED, "kernel does not fit on an SM");
  const int grid = std::max(1, std::min(d->n_cells, per_sm * sms));
  // the counter must start at zero; the per-cell words are overwritten by every cell
  MSFEM_CUDA(cudaMemsetAsync(p.queue, 0, sizeof(unsigned int), s));
  void *args[] = {&p};
  MSFEM_CUDA(cudaLaunchKernel(L.fn, dim3(grid), dim3(L.nt), args, L.smem, s));
  return MSFEM_OK;
}

const char *msfem_version(void) { return "msfem_gpu 0.1 (sm_103a)"; }

int msfem_last_error(char *buf, size_t len) {
  if (!buf || len == 0) return MSFEM_ERR_INVALID_ARG;
  std::snprintf(buf, len, "%s", g_last_error.c_str());
  return MSFEM_OK;
}

int msfem_create(msfem_handle **handle, int device) {
  if (!handle) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  *handle = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return fail(MSFEM_ERR_NO_DEVICE, "CUDA device " + std::to_string(device) + " not available");
  cudaDeviceProp prop;
  MSFEM_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3)
    return fail(MSFEM_ERR_NO_DEVICE, std::string("device is sm_") + std::to_string(prop.major) +
                                         std::to_string(prop.minor) + ", the library is compiled for sm_103a");
  MSFEM_CUDA(cudaSetDevice(device));
  msfem_handle *h = new msfem_handle();
  h->device = device;
  h->sm_count = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    if (h->side_stream) cudaStreamDestroy(h->side_stream);
    delete h;
    return fail(MSFEM_ERR_CUDA, "stream/event creation failed");
  }
  h->stream = h->own_stream;
  *handle = h;
  return MSFEM_OK;
}

int msfem_destroy(msfem_handle *h) {
  if (!h) return MSFEM_OK;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  cudaStreamSynchronize(h->side_stream);
  DevBuf *bufs[] = {&h->corners, &h->nfine, &h->order, &h->queue, &h->qp, &h->qpoff, &h->fqp, &h->fqpoff, &h->warm,
                    &h->boff, &h->modes, &h->spheres, &h->sgrid_start, &h->sgrid_ids,
                    &h->M, &h->F, &h->basis, &h->status, &h->iters, &h->relres, &h->refine,
                    &h->work};
  for (DevBuf *b : bufs) b->release();
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  if (h->side_stream) cudaStreamDestroy(h->side_stream);
  delete h;
  return MSFEM_OK;
}

int msfem_graph_info(msfem_handle *h, int64_t *captures, int64_t *replays) {
  if (!h) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  if (captures) *captures = h->graph_captures;
  if (replays) *replays = h->graph_launches;
  return MSFEM_OK;
}

int msfem_set_stream(msfem_handle *h, void *stream) {
  if (!h) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
  return MSFEM_OK;
}

int64_t msfem_tabulated_size(const msfem_batch_desc *d, int32_t ncomp) {
  if (!d || (d->dim != 2 && d->dim != 3) || d->n_cells < 0) return -1;
  const int nq = 1 << d->dim;
  if (!d->n_fine_per_cell) return (int64_t)d->n_cells * ncomp * nq * ipow(d->n_fine, d->dim);
  if (d->memory == MSFEM_MEM_DEVICE) return -1;  // sizes live on the device
  int64_t s = 0;
  for (int c = 0; c < d->n_cells; ++c) s += (int64_t)ncomp * nq * ipow(d->n_fine_per_cell[c], d->dim);
  return s;
}

int msfem_tabulate_coefficient(msfem_handle *h, const msfem_batch_desc *d, int32_t ncomp,
                               double *qp_values) {
  if (!h) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  int rc = validate(d);
  if (rc) return rc;
  if (d->coef.kind == MSFEM_COEF_TABULATED)
    return fail(MSFEM_ERR_INVALID_ARG, "coefficient is already tabulated");
  const int full = d->dim == 2 ? 3 : 6;
  if (ncomp != 1 && ncomp != full) return fail(MSFEM_ERR_INVALID_ARG, "ncomp must be 1 or d(d+1)/2");
  if (d->n_cells > 0 && !qp_values) return fail(MSFEM_ERR_INVALID_ARG, "qp_values is NULL");
  MSFEM_CUDA(cudaSetDevice(h->device));
  std::vector<int32_t> nf;
  if ((rc = host_nfine(h, d, nf))) return rc;
  const bool dev = d->memory == MSFEM_MEM_DEVICE;
  const int nv = 1 << d->dim;
  int64_t h2d = 0;
  int launches = 0;
  const double *corners = nullptr;
  const int32_t *nfd = nullptr;
  if ((rc = upload<double>(h, h->corners, d->corners, (size_t)d->n_cells * nv * d->dim, dev, &corners, &h2d))) return rc;
  if (d->n_fine_per_cell)
    if ((rc = upload<int32_t>(h, h->nfine, d->n_fine_per_cell, (size_t)d->n_cells, dev, &nfd, &h2d))) return rc;
  std::vector<int64_t> off;
  const int64_t *offd = nullptr;
  int64_t total = (int64_t)d->n_cells * ncomp * nv * ipow(d->n_fine, d->dim);
  if (d->n_fine_per_cell) {
    off.resize(d->n_cells);
    total = 0;
    for (int c = 0; c < d->n_cells; ++c) {
      off[c] = total;
      total += (int64_t)ncomp * nv * ipow(nf[c], d->dim);
    }
    if ((rc = upload<int64_t>(h, h->qpoff, off.data(), off.size(), false, &offd, &h2d))) return rc;
  }
  double *out = qp_values;
  if (!dev) {
    MSFEM_CUDA(h->qp.ensure(sizeof(double) * std::max<int64_t>(1, total)));
    out = h->qp.as<double>();
  }
  if ((rc = run_tabulate(h, d, nf, corners, nfd, ncomp, out, offd, &h2d, &launches))) return rc;
  if (!dev && total > 0)
    MSFEM_CUDA(cudaMemcpyAsync(qp_values, out, sizeof(double) * total, cudaMemcpyDeviceToHost, h->stream));
  MSFEM_CUDA(cudaStreamSynchronize(h->stream));
  return MSFEM_OK;
}

}  // extern "C"

// ===========================================================================
// Learned warm start: network object, training and inference
// ===========================================================================
namespace msfem {

// Node features of N = 32 cells from the tabulated coefficient:
// the tensor averaged over the node's fine cells (4 Gauss points each),
// then (log a11, a12 / sqrt(a11 a22), log a22).  The inputs are FP64; the
// arithmetic is FP32 (the features feed a BF16 network, and FP64 logarithms
// at GB300's FP64 rate would cost more than the network itself).  Two
// passes per cell: the Gauss-point sums of every fine cell (coalesced
// reads of the component-major table, each value read once) into shared
// memory, then the node averages.
__global__ void __launch_bounds__(256) features_kernel(const double *__restrict__ qp, int ncomp,
                                                       const int64_t *__restrict__ qp_offset, int n_cells,
                                                       float *__restrict__ feat) {
  constexpr int N = 32, n = 33, nfc = N * N;
  __shared__ float csum[3][nfc];
  const int cell = blockIdx.x;
  if (cell >= n_cells) return;
  const double *tab = qp + (qp_offset ? qp_offset[cell] : (int64_t)cell * ncomp * 4 * nfc);
  for (int i = threadIdx.x; i < ncomp * nfc; i += blockDim.x) {
    const int c = i / nfc, fc = i - c * nfc;
    const double *t = tab + (int64_t)c * 4 * nfc + fc;
    csum[c][fc] = (float)((__ldg(t) + __ldg(t + nfc)) + (__ldg(t + 2 * nfc) + __ldg(t + 3 * nfc)));
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
    const int ix = k % n, iy = k / n;
    float a[3] = {0.0f, 0.0f, 0.0f};
    int cnt = 0;
    for (int dy = -1; dy <= 0; ++dy)
      for (int dx = -1; dx <= 0; ++dx) {
        const int cx = ix + dx, cy = iy + dy;
        if (cx < 0 || cy < 0 || cx >= N || cy >= N) continue;
        const int fc = cx + N * cy;
        ++cnt;
        for (int c = 0; c < ncomp; ++c) a[c] += csum[c][fc];
      }
    if (ncomp == 1) a[2] = a[0];
    const float sc = 1.0f / (4.0f * (float)cnt);
    const float a11 = a[0] * sc, a12 = ncomp == 1 ? 0.0f : a[1] * sc, a22 = a[2] * sc;
    float *o = feat + (int64_t)cell * 3 * n * n + k;
    o[0] = logf(a11);
    o[n * n] = a12 * rsqrtf(a11 * a22);
    o[2 * n * n] = logf(a22);
  }
}

// Fine-scale solution of every cell, u = sum_i w_i phi_i over its nodes
// (set_global_weights and the per-cell reconstruction of
// diffusion_problem_basis.tpp:352-377).  One CTA per cell (grid-stride over
// cells), coalesced along the nodes; HBM-bound: 2^d + 1 doubles per node.
__global__ void reconstruct_kernel(int dim, int n_cells, int n_uniform, const int32_t *__restrict__ n_fine,
                                   const int64_t *__restrict__ boff, const double *__restrict__ basis,
                                   const double *__restrict__ w, double *__restrict__ u) {
  const int nv = 1 << dim;
  for (int cell = blockIdx.x; cell < n_cells; cell += gridDim.x) {
    const int n = (n_fine ? n_fine[cell] : n_uniform) + 1;
    const int nn = dim == 2 ? n * n : n * n * n;
    const int64_t b0 = boff ? boff[cell] : (int64_t)cell * nv * nn;
    const int64_t u0 = b0 / nv;
    double wc[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) wc[i] = i < nv ? __ldg(w + (int64_t)cell * nv + i) : 0.0;
    for (int k = threadIdx.x; k < nn; k += blockDim.x) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (i < nv) s = fma(wc[i], __ldg(basis + b0 + (int64_t)i * nn + k), s);
      u[u0 + k] = s;
    }
  }
}

// Warm basis = Q1 hat + predicted correction, FP64 [cell][4][33*33].
__global__ void compose_warm_kernel(const float *__restrict__ delta, int n_cells, double *__restrict__ warm) {
  constexpr int n = 33, nn = n * n;
  const long total = (long)n_cells * 4 * nn;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int k = (int)(i % nn), b = (int)((i / nn) % 4);
    const double tx = (k % n) / 32.0, ty = (k / n) / 32.0;
    const double hx = (b & 1) ? tx : 1.0 - tx, hy = (b & 2) ? ty : 1.0 - ty;
    warm[i] = hx * hy + (double)delta[i];
  }
}

// Training targets delta = phi - Q1 hat (inverse of compose_warm_kernel).
__global__ void targets_kernel(const double *__restrict__ basis, int n_cells, float *__restrict__ delta) {
  constexpr int n = 33, nn = n * n;
  const long total = (long)n_cells * 4 * nn;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int k = (int)(i % nn), b = (int)((i / nn) % 4);
    const double tx = (k % n) / 32.0, ty = (k / n) / 32.0;
    const double hx = (b & 1) ? tx : 1.0 - tx, hy = (b & 2) ? ty : 1.0 - ty;
    delta[i] = (float)(basis[i] - hx * hy);
  }
}

}  // namespace msfem

struct msfem_surrogate {
  msfem_handle *h = nullptr;
  int capacity = 0;
  int64_t step = 0;
  DevBuf params, grads, m, v, loss;
  DevBuf wf[msfem::cnn::kLayers], wt[msfem::cnn::kLayers], bpad[msfem::cnn::kLayers];
  DevBuf act[msfem::cnn::kLayers + 1];  // act[0] input, act[1..5] hidden, act[6] FP32 prediction
  DevBuf ga, gb;                        // gradient ping-pong (channel-blocked bf16)
  DevBuf tc_err;                        // int: timeout code of the tensor-core convolution (0 = none)
};

namespace {

using bf16 = __nv_bfloat16;
namespace cn = msfem::cnn;

// One 3x3 convolution layer on the tcgen05 tensor cores (cnn_tc.cu).
template <int CIN, int COUT, int EPI>
int launch_conv(msfem_surrogate *s, int B, const bf16 *X, const bf16 *W, const float *bias, const bf16 *mask,
                void *out, int cout_real, int dil) {
  const cn::ConvCtx ctx{s->h->stream, s->h->device, s->h->sm_count, s->tc_err.as<int>()};
  std::string msg;
  const int rc = cn::conv_tc(ctx, CIN, COUT, EPI, B, X, W, bias, mask, out, cout_real, dil, &msg);
  return rc ? fail(rc, msg) : MSFEM_OK;
}

// After a synchronisation: report (and clear) a timeout of the tensor-core
// convolution's pipeline.
int surrogate_check(msfem_surrogate *s) {
  int code = 0;
  MSFEM_CUDA(cudaMemcpy(&code, s->tc_err.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  if (!code) return MSFEM_OK;
  MSFEM_CUDA(cudaMemset(s->tc_err.ptr, 0, sizeof(int)));
  return fail(MSFEM_ERR_CUDA, std::string("tensor-core convolution timed out in its ") +
                                  (code == 1 ? "window loads (TMA)" : code == 2 ? "MMA issue" : "epilogue"));
}

// Weight and bias gradient of one layer on the tcgen05 tensor cores (cnn_tc.cu).
template <int XC, int GC>
int launch_wgrad(msfem_surrogate *s, int B, const bf16 *X, const bf16 *G, int cin_real, int cout_real, float *dW,
                 float *db, int dil) {
  const cn::ConvCtx ctx{s->h->stream, s->h->device, s->h->sm_count, s->tc_err.as<int>()};
  std::string msg;
  const int rc = cn::wgrad_tc(ctx, XC, GC, B, X, G, cin_real, cout_real, dW, db, dil, &msg);
  return rc ? fail(rc, msg) : MSFEM_OK;
}

int surrogate_reserve(msfem_surrogate *s, int B) {
  if (B <= s->capacity) return MSFEM_OK;
  for (int l = 0; l < cn::kLayers; ++l)
    MSFEM_CUDA(s->act[l].ensure(sizeof(bf16) * (size_t)B * cn::kPix * cn::pad_ch(l)));
  MSFEM_CUDA(s->act[cn::kLayers].ensure(sizeof(float) * (size_t)B * 4 * cn::kPix));
  MSFEM_CUDA(s->ga.ensure(sizeof(bf16) * (size_t)B * cn::kPix * 32));
  MSFEM_CUDA(s->gb.ensure(sizeof(bf16) * (size_t)B * cn::kPix * 32));
  s->capacity = B;
  return MSFEM_OK;
}

int surrogate_pack(msfem_surrogate *s) {
  cudaStream_t st = s->h->stream;
  for (int l = 0; l < cn::kLayers; ++l) {
    const size_t nw = (size_t)cn::pad_ch(l + 1) * 9 * cn::pad_ch(l);
    MSFEM_CUDA(s->wf[l].ensure(sizeof(bf16) * nw));
    MSFEM_CUDA(s->wt[l].ensure(sizeof(bf16) * nw));
    MSFEM_CUDA(s->bpad[l].ensure(sizeof(float) * cn::pad_ch(l + 1)));
    cn::pack_layer_kernel<<<64, 256, 0, st>>>(s->params.as<float>(), l, s->wf[l].as<bf16>(), s->wt[l].as<bf16>(),
                                              s->bpad[l].as<float>());
    MSFEM_CUDA(cudaGetLastError());
  }
  return MSFEM_OK;
}

// Forward pass of B images; the prediction goes to `out` (FP32 NCHW, 4 ch).
int surrogate_forward(msfem_surrogate *s, const float *features, int B, float *out) {
  cudaStream_t st = s->h->stream;
  int rc;
  if ((rc = surrogate_reserve(s, B))) return rc;
  if (!out || !features) return fail(MSFEM_ERR_INVALID_ARG, "surrogate forward: NULL buffer");
  cn::features_to_blocked_kernel<<<std::max(1, std::min(B * 4, 4096)), 256, 0, st>>>(features, B, s->act[0].as<bf16>());
  MSFEM_CUDA(cudaGetLastError());
  if ((rc = launch_conv<16, 32, cn::EPI_RELU_BF16>(s, B, s->act[0].as<bf16>(), s->wf[0].as<bf16>(),
                                                  s->bpad[0].as<float>(), nullptr, s->act[1].ptr, 32,
                                                  cn::dilation(0)))) return rc;
  for (int l = 1; l < 5; ++l)
    if ((rc = launch_conv<32, 32, cn::EPI_RELU_BF16>(s, B, s->act[l].as<bf16>(), s->wf[l].as<bf16>(),
                                                    s->bpad[l].as<float>(), nullptr, s->act[l + 1].ptr, 32,
                                                    cn::dilation(l))))
      return rc;
  return launch_conv<32, 16, cn::EPI_F32_NCHW>(s, B, s->act[5].as<bf16>(), s->wf[5].as<bf16>(),
                                              s->bpad[5].as<float>(), nullptr, out, 4, cn::dilation(5));
}

// Loss and gradients of one batch into s->grads (FP32) and s->loss (double).
int surrogate_backward(msfem_surrogate *s, const float *features, const float *targets, int B) {
  cudaStream_t st = s->h->stream;
  int rc;
  // reserve first: the prediction buffer must exist before its pointer is taken
  if ((rc = surrogate_reserve(s, B))) return rc;
  if ((rc = surrogate_forward(s, features, B, s->act[cn::kLayers].as<float>()))) return rc;
  MSFEM_CUDA(cudaMemsetAsync(s->grads.ptr, 0, sizeof(float) * cn::kParams, st));
  MSFEM_CUDA(cudaMemsetAsync(s->loss.ptr, 0, sizeof(double), st));
  const float scale = 1.0f / (float)((double)B * 4 * (cn::kH - 2) * (cn::kW - 2));
  cn::mse_loss_kernel<<<std::max(1, std::min(B * 4, 4096)), 256, 0, st>>>(
      s->act[cn::kLayers].as<float>(), targets, B, scale, s->ga.as<bf16>(), s->loss.as<double>());
  MSFEM_CUDA(cudaGetLastError());
  float *G = s->grads.as<float>();
  auto dW = [&](int l) { return G + cn::param_offset(l); };
  auto db = [&](int l) { return G + cn::param_offset(l) + (long)cn::real_ch(l + 1) * cn::real_ch(l) * 9; };
  // layer 6: g (16 ch) in ga
  if ((rc = launch_wgrad<32, 16>(s, B, s->act[5].as<bf16>(), s->ga.as<bf16>(), 32, 4, dW(5), db(5),
                                 cn::dilation(5)))) return rc;
  if ((rc = launch_conv<16, 32, cn::EPI_MASK_BF16>(s, B, s->ga.as<bf16>(), s->wt[5].as<bf16>(), nullptr,
                                                  s->act[5].as<bf16>(), s->gb.ptr, 32, cn::dilation(5)))) return rc;
  bf16 *g = s->gb.as<bf16>(), *gn = s->ga.as<bf16>();
  for (int l = 4; l >= 1; --l) {
    if ((rc = launch_wgrad<32, 32>(s, B, s->act[l].as<bf16>(), g, 32, 32, dW(l), db(l), cn::dilation(l))))
      return rc;
    if ((rc = launch_conv<32, 32, cn::EPI_MASK_BF16>(s, B, g, s->wt[l].as<bf16>(), nullptr, s->act[l].as<bf16>(),
                                                    gn, 32, cn::dilation(l)))) return rc;
    std::swap(g, gn);
  }
  return launch_wgrad<16, 32>(s, B, s->act[0].as<bf16>(), g, 3, 32, dW(0), db(0), cn::dilation(0));
}

// The warm start inside msfem_run_batch: features -> prediction -> Q1 + delta.
int surrogate_warm_start(msfem_handle *h, msfem::KernelParams &p, int nc, int *launches) {
  msfem_surrogate *s = h->surrogate;
  const int n = 33 * 33;
  MSFEM_CUDA(h->feat.ensure(sizeof(float) * (size_t)nc * 3 * n));
  MSFEM_CUDA(h->delta.ensure(sizeof(float) * (size_t)nc * 4 * n));
  MSFEM_CUDA(h->warm_pred.ensure(sizeof(double) * (size_t)nc * 4 * n));
  msfem::features_kernel<<<nc, 256, 0, h->stream>>>(p.qp_values, p.ncomp, p.qp_offset, nc, h->feat.as<float>());
  MSFEM_CUDA(cudaGetLastError());
  const int chunk = 4096;
  int rc;
  for (int c0 = 0; c0 < nc; c0 += chunk) {
    const int b = std::min(chunk, nc - c0);
    if ((rc = surrogate_forward(s, h->feat.as<float>() + (size_t)c0 * 3 * n, b,
                                h->delta.as<float>() + (size_t)c0 * 4 * n))) return rc;
    *launches += 7;
  }
  msfem::compose_warm_kernel<<<std::min(nc * 4, 8192), 256, 0, h->stream>>>(h->delta.as<float>(), nc,
                                                                             h->warm_pred.as<double>());
  MSFEM_CUDA(cudaGetLastError());
  *launches += 2;
  p.warm_basis = h->warm_pred.as<double>();
  return MSFEM_OK;
}

}  // namespace

extern "C" {

int64_t msfem_surrogate_param_count(void) { return cn::kParams; }

int msfem_surrogate_create(msfem_handle *h, uint64_t seed, msfem_surrogate **out) {
  if (!h || !out) return fail(MSFEM_ERR_INVALID_ARG, "handle and output are required");
  MSFEM_CUDA(cudaSetDevice(h->device));
  auto *s = new msfem_surrogate();
  s->h = h;
  // He-uniform weights (last layer scaled down so the first predictions are
  // near zero), zero biases; SplitMix64 stream
  std::vector<float> w(cn::kParams, 0.0f);
  uint64_t state = seed;
  auto next = [&]() {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < cn::kLayers; ++l) {
    const int cin = cn::real_ch(l), cout = cn::real_ch(l + 1);
    const double bound = std::sqrt(6.0 / (cin * 9.0)) * (l == cn::kLayers - 1 ? 0.1 : 1.0);
    float *W = w.data() + cn::param_offset(l);
    for (long i = 0; i < (long)cout * cin * 9; ++i) W[i] = (float)((2.0 * next() - 1.0) * bound);
  }
  int rc = MSFEM_OK;
  if (s->params.ensure(sizeof(float) * cn::kParams) != cudaSuccess || s->grads.ensure(sizeof(float) * cn::kParams) != cudaSuccess ||
      s->m.ensure(sizeof(float) * cn::kParams) != cudaSuccess || s->v.ensure(sizeof(float) * cn::kParams) != cudaSuccess ||
      s->loss.ensure(sizeof(double)) != cudaSuccess || s->tc_err.ensure(sizeof(int)) != cudaSuccess)
    rc = fail(MSFEM_ERR_OUT_OF_MEMORY, "surrogate allocation failed");
  if (!rc && cudaMemsetAsync(s->tc_err.ptr, 0, sizeof(int), h->stream) != cudaSuccess)
    rc = fail(MSFEM_ERR_CUDA, "surrogate state init failed");
  if (!rc && cudaMemcpyAsync(s->params.ptr, w.data(), sizeof(float) * cn::kParams, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    rc = fail(MSFEM_ERR_CUDA, "surrogate parameter upload failed");
  if (!rc && (cudaMemsetAsync(s->m.ptr, 0, sizeof(float) * cn::kParams, h->stream) != cudaSuccess ||
              cudaMemsetAsync(s->v.ptr, 0, sizeof(float) * cn::kParams, h->stream) != cudaSuccess))
    rc = fail(MSFEM_ERR_CUDA, "surrogate state init failed");
  if (!rc) rc = surrogate_pack(s);
  if (!rc && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = fail(MSFEM_ERR_CUDA, "surrogate init failed");
  if (rc) {
    msfem_surrogate_destroy(s);
    return rc;
  }
  *out = s;
  return MSFEM_OK;
}

int msfem_surrogate_destroy(msfem_surrogate *s) {
  if (!s) return MSFEM_OK;
  cudaSetDevice(s->h->device);
  cudaStreamSynchronize(s->h->stream);
  if (s->h->surrogate == s) s->h->surrogate = nullptr;
  DevBuf *bufs[] = {&s->params, &s->grads, &s->m, &s->v, &s->loss, &s->ga, &s->gb, &s->tc_err};
  for (DevBuf *b : bufs) b->release();
  for (int l = 0; l < cn::kLayers; ++l) {
    s->wf[l].release();
    s->wt[l].release();
    s->bpad[l].release();
  }
  for (auto &a : s->act) a.release();
  delete s;
  return MSFEM_OK;
}

int msfem_surrogate_set_params(msfem_surrogate *s, const float *params) {
  if (!s || !params) return fail(MSFEM_ERR_INVALID_ARG, "surrogate and params are required");
  MSFEM_CUDA(cudaSetDevice(s->h->device));
  MSFEM_CUDA(cudaMemcpyAsync(s->params.ptr, params, sizeof(float) * cn::kParams, cudaMemcpyHostToDevice, s->h->stream));
  int rc = surrogate_pack(s);
  if (rc) return rc;
  MSFEM_CUDA(cudaStreamSynchronize(s->h->stream));
  return MSFEM_OK;
}

int msfem_surrogate_get_params(msfem_surrogate *s, float *params) {
  if (!s || !params) return fail(MSFEM_ERR_INVALID_ARG, "surrogate and params are required");
  MSFEM_CUDA(cudaSetDevice(s->h->device));
  MSFEM_CUDA(cudaMemcpyAsync(params, s->params.ptr, sizeof(float) * cn::kParams, cudaMemcpyDeviceToHost, s->h->stream));
  MSFEM_CUDA(cudaStreamSynchronize(s->h->stream));
  return MSFEM_OK;
}

int msfem_surrogate_features(msfem_handle *h, const msfem_batch_desc *d, float *features) {
  if (!h) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  int rc = validate(d);
  if (rc) return rc;
  if (d->dim != 2 || d->n_fine != 32 || d->n_fine_per_cell || d->coef.kind != MSFEM_COEF_TABULATED ||
      d->memory != MSFEM_MEM_DEVICE)
    return fail(MSFEM_ERR_UNSUPPORTED, "surrogate features: 2D, N = 32, TABULATED coefficient in device memory");
  if (d->n_cells == 0) return MSFEM_OK;
  MSFEM_CUDA(cudaSetDevice(h->device));
  msfem::features_kernel<<<d->n_cells, 256, 0, h->stream>>>(d->coef.qp_values, d->coef.ncomp, d->coef.qp_offset,
                                                             d->n_cells, features);
  MSFEM_CUDA(cudaGetLastError());
  MSFEM_CUDA(cudaStreamSynchronize(h->stream));
  return MSFEM_OK;
}

int msfem_surrogate_targets(msfem_handle *h, const double *basis, int32_t n, float *delta) {
  if (!h || n < 0 || (n > 0 && (!basis || !delta))) return fail(MSFEM_ERR_INVALID_ARG, "bad surrogate_targets arguments");
  if (n == 0) return MSFEM_OK;
  MSFEM_CUDA(cudaSetDevice(h->device));
  msfem::targets_kernel<<<std::min(n * 4, 8192), 256, 0, h->stream>>>(basis, n, delta);
  MSFEM_CUDA(cudaGetLastError());
  MSFEM_CUDA(cudaStreamSynchronize(h->stream));
  return MSFEM_OK;
}

int msfem_surrogate_predict(msfem_surrogate *s, const float *features, int32_t n, float *delta) {
  if (!s || (n > 0 && (!features || !delta))) return fail(MSFEM_ERR_INVALID_ARG, "bad surrogate_predict arguments");
  MSFEM_CUDA(cudaSetDevice(s->h->device));
  const int chunk = 4096;
  for (int c0 = 0; c0 < n; c0 += chunk) {
    const int b = std::min(chunk, n - c0);
    int rc = surrogate_forward(s, features + (size_t)c0 * 3 * cn::kPix, b, delta + (size_t)c0 * 4 * cn::kPix);
    if (rc) return rc;
  }
  MSFEM_CUDA(cudaStreamSynchronize(s->h->stream));
  return surrogate_check(s);
}

int msfem_surrogate_gradients(msfem_surrogate *s, const float *features, const float *targets, int32_t batch,
                              float *grads_host, double *loss) {
  if (!s || batch < 1 || !features || !targets) return fail(MSFEM_ERR_INVALID_ARG, "bad surrogate_gradients arguments");
  MSFEM_CUDA(cudaSetDevice(s->h->device));
  int rc = surrogate_backward(s, features, targets, batch);
  if (rc) return rc;
  if (grads_host)
    MSFEM_CUDA(cudaMemcpyAsync(grads_host, s->grads.ptr, sizeof(float) * cn::kParams, cudaMemcpyDeviceToHost, s->h->stream));
  double l = 0.0;
  MSFEM_CUDA(cudaMemcpyAsync(&l, s->loss.ptr, sizeof(double), cudaMemcpyDeviceToHost, s->h->stream));
  MSFEM_CUDA(cudaStreamSynchronize(s->h->stream));
  if (loss) *loss = l;
  return surrogate_check(s);
}

int msfem_surrogate_train_step(msfem_surrogate *s, const float *features, const float *targets, int32_t batch,
                               float lr, double *loss) {
  if (!s || batch < 1 || !features || !targets || !(lr > 0.0f))
    return fail(MSFEM_ERR_INVALID_ARG, "bad surrogate_train_step arguments");
  MSFEM_CUDA(cudaSetDevice(s->h->device));
  int rc = surrogate_backward(s, features, targets, batch);
  if (rc) return rc;
  s->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.0f - std::pow(b1, (float)s->step), bc2 = 1.0f - std::pow(b2, (float)s->step);
  cn::adam_kernel<<<64, 256, 0, s->h->stream>>>(s->params.as<float>(), s->grads.as<float>(), s->m.as<float>(),
                                                s->v.as<float>(), cn::kParams, lr, b1, b2, 1e-8f, bc1, bc2);
  MSFEM_CUDA(cudaGetLastError());
  if ((rc = surrogate_pack(s))) return rc;
  if (loss) {
    MSFEM_CUDA(cudaMemcpyAsync(loss, s->loss.ptr, sizeof(double), cudaMemcpyDeviceToHost, s->h->stream));
    MSFEM_CUDA(cudaStreamSynchronize(s->h->stream));
    return surrogate_check(s);
  }
  return MSFEM_OK;
}

int msfem_attach_surrogate(msfem_handle *h, msfem_surrogate *s) {
  if (!h) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  if (s && s->h != h) return fail(MSFEM_ERR_INVALID_ARG, "surrogate belongs to another handle");
  h->surrogate = s;
  return MSFEM_OK;
}

}  // extern "C"

namespace {

// msfem_run_batch with an optional forced launch choice (autotuning).
// Device inputs of a batch (corners, per-cell N, basis offsets, the
// size-sorted work queue and the coefficient, tabulated on the device for the
// FOURIER and SPHERES kinds) into the kernel parameters; basis_total is the
// length of the basis-output layout.
int prepare_inputs(msfem_handle *h, const msfem_batch_desc *d, const std::vector<int32_t> &nf,
                   KernelParams &p, int64_t &basis_total, int64_t &h2d, int &launches) {
  const int dim = d->dim, nv = 1 << dim, nc = d->n_cells;
  const bool dev = d->memory == MSFEM_MEM_DEVICE;
  int rc = 0;
  const double *corners = nullptr;
  const int32_t *nfd = nullptr;
  if ((rc = upload<double>(h, h->corners, d->corners, (size_t)nc * nv * dim, dev, &corners, &h2d))) return rc;
  if (d->n_fine_per_cell)
    if ((rc = upload<int32_t>(h, h->nfine, d->n_fine_per_cell, (size_t)nc, dev, &nfd, &h2d))) return rc;
  // per-cell basis offsets (uneven N) and the size-sorted work queue
  std::vector<int64_t> boff;
  const int64_t *boffd = nullptr;
  const int32_t *orderd = nullptr;
  basis_total = (int64_t)nc * nv * ipow(d->n_fine + 1, dim);
  if (d->n_fine_per_cell) {
    boff.resize(nc);
    basis_total = 0;
    for (int c = 0; c < nc; ++c) {
      boff[c] = basis_total;
      basis_total += (int64_t)nv * ipow(nf[c] + 1, dim);
    }
    if ((rc = upload<int64_t>(h, h->boff, boff.data(), boff.size(), false, &boffd, &h2d))) return rc;
    // largest cells first (counting sort on N, stable)
    std::vector<int32_t> order(nc);
    std::vector<int> cnt(MSFEM_MAX_N_2D + 2, 0);
    for (int c = 0; c < nc; ++c) cnt[nf[c]]++;
    std::vector<int> pos(MSFEM_MAX_N_2D + 2, 0);
    int acc = 0;
    for (int v = MSFEM_MAX_N_2D; v >= 1; --v) { pos[v] = acc; acc += cnt[v]; }
    for (int c = 0; c < nc; ++c) order[pos[nf[c]]++] = c;
    if ((rc = upload<int32_t>(h, h->order, order.data(), order.size(), false, &orderd, &h2d))) return rc;
  }
  // coefficient
  p = KernelParams{};
  p.dim = dim;
  p.n_cells = nc;
  p.n_fine_uniform = d->n_fine;
  p.corners = corners;
  p.n_fine = nfd;
  p.order = orderd;
  p.f_value = d->f_value;
  p.coef_kind = d->coef.kind;
  p.ncomp = d->coef.ncomp;
  for (int k = 0; k < 8; ++k) p.cparams[k] = d->coef.params[k];
  if (p.coef_kind == MSFEM_COEF_REFERENCE) reference_rrt(dim, p.cparams);
  if (d->coef.kind == MSFEM_COEF_TABULATED) {
    int64_t total = 0;
    std::vector<int64_t> off;
    if (d->n_fine_per_cell || d->coef.qp_offset) {
      off.resize(nc);
      for (int c = 0; c < nc; ++c) {
        off[c] = total;
        total += (int64_t)d->coef.ncomp * nv * ipow(cell_N(d, nf, c), dim);
      }
    } else {
      total = (int64_t)nc * d->coef.ncomp * nv * ipow(d->n_fine, dim);
    }
    if (d->coef.qp_offset) {
      // caller-provided offsets: data extent = max offset + block
      const int64_t *qo = d->coef.qp_offset;
      std::vector<int64_t> hq(nc);
      if (dev) {
        MSFEM_CUDA(cudaMemcpyAsync(hq.data(), qo, sizeof(int64_t) * nc, cudaMemcpyDeviceToHost, h->stream));
        MSFEM_CUDA(cudaStreamSynchronize(h->stream));
      } else {
        std::memcpy(hq.data(), qo, sizeof(int64_t) * nc);
      }
      total = 0;
      for (int c = 0; c < nc; ++c)
        total = std::max(total, hq[c] + (int64_t)d->coef.ncomp * nv * ipow(cell_N(d, nf, c), dim));
      off = hq;
    }
    const double *qp = nullptr;
    if ((rc = upload<double>(h, h->qp, d->coef.qp_values, (size_t)total, dev, &qp, &h2d))) return rc;
    p.qp_values = qp;
    if (!off.empty()) {
      const int64_t *od = nullptr;
      if ((rc = upload<int64_t>(h, h->qpoff, off.data(), off.size(), false, &od, &h2d))) return rc;
      p.qp_offset = od;
    }
  } else if (d->coef.kind == MSFEM_COEF_FOURIER || d->coef.kind == MSFEM_COEF_SPHERES ||
             d->warm_start == MSFEM_WARM_SURROGATE) {
    // tabulate on the device first, then run the tabulated path
    const int ncomp = (d->coef.kind == MSFEM_COEF_SPHERES || dim == 3) ? 1 : 3;
    std::vector<int64_t> off;
    int64_t total = (int64_t)nc * ncomp * nv * ipow(d->n_fine, dim);
    const int64_t *od = nullptr;
    if (d->n_fine_per_cell) {
      off.resize(nc);
      total = 0;
      for (int c = 0; c < nc; ++c) {
        off[c] = total;
        total += (int64_t)ncomp * nv * ipow(nf[c], dim);
      }
      if ((rc = upload<int64_t>(h, h->qpoff, off.data(), off.size(), false, &od, &h2d))) return rc;
    }
    MSFEM_CUDA(h->qp.ensure(sizeof(double) * std::max<int64_t>(1, total)));
    if ((rc = run_tabulate(h, d, nf, corners, nfd, ncomp, h->qp.as<double>(), od, &h2d, &launches))) return rc;
    p.coef_kind = MSFEM_COEF_TABULATED;
    p.ncomp = ncomp;
    p.qp_values = h->qp.as<double>();
    p.qp_offset = od;
  }
  // right-hand side at the Gauss points: blocks of 2^d N_c^d per cell
  p.f_qp = nullptr;
  p.f_qp_offset = nullptr;
  if (d->f_qp_values && nc > 0) {
    std::vector<int64_t> off;
    int64_t total = 0;
    if (d->f_qp_offset) {
      off.resize(nc);
      if (dev) {
        MSFEM_CUDA(cudaMemcpyAsync(off.data(), d->f_qp_offset, sizeof(int64_t) * nc, cudaMemcpyDeviceToHost,
                                   h->stream));
        MSFEM_CUDA(cudaStreamSynchronize(h->stream));
      } else {
        std::memcpy(off.data(), d->f_qp_offset, sizeof(int64_t) * nc);
      }
      for (int c = 0; c < nc; ++c) {
        if (off[c] < 0) return fail(MSFEM_ERR_INVALID_ARG, "f_qp_offset[" + std::to_string(c) + "] < 0");
        total = std::max(total, off[c] + (int64_t)nv * ipow(cell_N(d, nf, c), dim));
      }
    } else if (d->n_fine_per_cell) {
      off.resize(nc);
      for (int c = 0; c < nc; ++c) {
        off[c] = total;
        total += (int64_t)nv * ipow(nf[c], dim);
      }
    } else {
      total = (int64_t)nc * nv * ipow(d->n_fine, dim);
    }
    const double *fq = nullptr;
    if ((rc = upload<double>(h, h->fqp, d->f_qp_values, (size_t)total, dev, &fq, &h2d))) return rc;
    p.f_qp = fq;
    if (!off.empty()) {
      const int64_t *od = nullptr;
      if (d->f_qp_offset && dev) {
        od = d->f_qp_offset;
      } else if ((rc = upload<int64_t>(h, h->fqpoff, off.data(), off.size(), false, &od, &h2d))) {
        return rc;
      }
      p.f_qp_offset = od;
    }
  }
  p.basis_offset = boffd;
  return MSFEM_OK;
}

int run_batch_impl(msfem_handle *h, const msfem_batch_desc *d, double *M, double *F,
                   double *basis, int32_t *cell_status, int32_t *iterations,
                   msfem_stats *stats, const Tune *force) {
  const auto t_start = std::chrono::steady_clock::now();
  if (!h) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  int rc = validate(d);
  if (rc) return rc;
  if (d->n_cells > 0 && (!M || !F)) return fail(MSFEM_ERR_INVALID_ARG, "M and F are required");
  MSFEM_CUDA(cudaSetDevice(h->device));
  const int dim = d->dim, nv = 1 << dim, nc = d->n_cells;
  const bool dev = d->memory == MSFEM_MEM_DEVICE;
  const bool mixed = d->precision == MSFEM_PREC_MIXED;
  std::vector<int32_t> nf;
  if ((rc = host_nfine(h, d, nf))) return rc;
  int nmax = d->n_fine;
  if (d->n_fine_per_cell) {
    nmax = 1;
    for (int c = 0; c < nc; ++c) nmax = std::max(nmax, nf[c]);
  }
  const std::vector<Launch> cands = candidates(dim, nmax, mixed);
  if (cands.empty())
    return fail(MSFEM_ERR_UNSUPPORTED, "no kernel for dim " + std::to_string(dim) + ", N " +
                                           std::to_string(nmax));
  Tune tn;
  if (force) {
    tn = *force;
  } else {
    auto it = h->tuning.find(tune_key(dim, nmax, mixed));
    if (it != h->tuning.end()) tn = it->second;
  }
  if (tn.variant < 0 || tn.variant >= (int)cands.size()) tn.variant = 0;
  const Launch L = cands[tn.variant];
  int64_t h2d = 0, d2h = 0;
  int launches = 0;

  // ---- inputs
  KernelParams p{};
  int64_t basis_total = 0;
  if ((rc = prepare_inputs(h, d, nf, p, basis_total, h2d, launches))) return rc;
  p.tol = d->tol;
  p.tol_abs = d->tol_absolute;
  p.maxit = d->maxit;
  p.check_interval = d->check_interval > 0 ? d->check_interval : tn.check_interval;
  p.inner_tol = tn.inner_tol;
  p.inner_maxit = std::max(1, std::min(d->maxit, 1000));
  p.max_refine = 40;
  p.cheb_ratio = tn.cheb_ratio;
  if (d->warm_start == MSFEM_WARM_USER) {
    const double *wb = nullptr;
    if ((rc = upload<double>(h, h->warm, d->warm_basis, (size_t)basis_total, dev, &wb, &h2d))) return rc;
    p.warm_basis = wb;
  }
  if (d->warm_start == MSFEM_WARM_SURROGATE && nc > 0) {
    if (!h->surrogate) return fail(MSFEM_ERR_INVALID_ARG, "MSFEM_WARM_SURROGATE: no surrogate attached");
    if (dim != 2 || d->n_fine_per_cell || d->n_fine != 32)
      return fail(MSFEM_ERR_UNSUPPORTED, "surrogate warm start: 2D cells with N = 32 only");
    if ((rc = surrogate_warm_start(h, p, nc, &launches))) return rc;
  }

  // ---- outputs
  auto out_ptr = [&](DevBuf &buf, void *user, size_t bytes) -> void * {
    if (dev && user) return user;
    if (buf.ensure(std::max<size_t>(bytes, 8)) != cudaSuccess) return nullptr;
    return buf.ptr;
  };
  p.M = (double *)out_ptr(h->M, M, sizeof(double) * nc * nv * nv);
  p.F = (double *)out_ptr(h->F, F, sizeof(double) * nc * nv);
  p.status = (int32_t *)out_ptr(h->status, cell_status, sizeof(int32_t) * nc);
  p.iters = (int32_t *)out_ptr(h->iters, iterations, sizeof(int32_t) * nc * nv);
  p.rel_res = (double *)out_ptr(h->relres, nullptr, sizeof(double) * nc);
  p.refinements = (int32_t *)out_ptr(h->refine, nullptr, sizeof(int32_t) * nc);
  p.basis = basis ? (double *)out_ptr(h->basis, basis, sizeof(double) * basis_total) : nullptr;
  if (!p.M || !p.F || !p.status || !p.iters || !p.rel_res || !p.refinements || (basis && !p.basis))
    return fail(MSFEM_ERR_OUT_OF_MEMORY, "device output allocation failed");
  MSFEM_CUDA(h->queue.ensure(2 * sizeof(unsigned int)));
  p.queue = h->queue.as<unsigned int>();

  // ---- size-class split (3D mixed, slab-cluster shape, uneven N).  The
  // cluster shape keeps a cell's inner CG in its CTAs' shared memory but
  // occupies whole groups of 8 SMs and is slow on small cells; the cells with
  // N > kSplitN (a prefix of the size-sorted order) go to the cluster launch,
  // the rest to one CTA per cell (the 2-CTA/SM shape) on the side stream, on
  // the SMs the clusters leave free.  Own queue counters, workspace slots
  // after the clusters'.
  constexpr int kSplitN = 16;
  int n_large = nc;
  const Launch *Ls = nullptr;
  if (dim == 3 && mixed && L.cluster > 1 && d->n_fine_per_cell && nc > 0) {
    n_large = 0;
    for (int c = 0; c < nc; ++c) n_large += nf[c] > kSplitN ? 1 : 0;
    for (const Launch &c : cands)
      if (c.cluster == 1 && c.minb == 2 && c.nt == 256) Ls = &c;
    if (!Ls || n_large == 0 || n_large == nc) {
      Ls = nullptr;
      n_large = nc;
    }
  }
  const bool split = Ls != nullptr;
  KernelParams ps = p;  // the small cells' launch
  if (split) {
    p.n_cells = n_large;
    ps.n_cells = nc - n_large;
    ps.order = p.order + n_large;
    ps.queue = p.queue + 1;
  }

  // ---- launch: persistent CTAs, size-sorted work queue
  if (L.smem > 0)
    MSFEM_CUDA(cudaFuncSetAttribute(L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
  int per_sm = 0;
  MSFEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, L.fn, L.nt, L.smem));
  if (per_sm < 1) return fail(MSFEM_ERR_UNSUPPORTED, "kernel does not fit on an SM");
  if (L.slot_bytes) per_sm = std::min(per_sm, L.minb);  // workspace slots per SM
  const int ncl_cells = p.n_cells;
  int grid = std::max(1, std::min(ncl_cells, per_sm * h->sm_count));
  int slots = grid;
  // thread-block clusters: as many co-resident clusters as the GPU holds,
  // one cell and one workspace slot per cluster
  cudaLaunchConfig_t ccfg = {};
  cudaLaunchAttribute cattr[1];
  int ncl = 0;
  if (L.cluster > 1) {
    if (L.cluster > 8)
      MSFEM_CUDA(cudaFuncSetAttribute(L.fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    ccfg.gridDim = dim3(L.cluster);
    ccfg.blockDim = dim3(L.nt);
    ccfg.dynamicSmemBytes = L.smem;
    ccfg.stream = h->stream;
    cattr[0].id = cudaLaunchAttributeClusterDimension;
    cattr[0].val.clusterDim.x = L.cluster;
    cattr[0].val.clusterDim.y = 1;
    cattr[0].val.clusterDim.z = 1;
    ccfg.attrs = cattr;
    ccfg.numAttrs = 1;
    MSFEM_CUDA(cudaOccupancyMaxActiveClusters(&ncl, L.fn, &ccfg));
    if (ncl < 1) return fail(MSFEM_ERR_UNSUPPORTED, "no cluster of this shape fits the GPU");
    slots = std::max(1, std::min(ncl_cells, ncl));
    grid = slots * L.cluster;
    ccfg.gridDim = dim3(grid);
  }
  // the small cells' launch: one CTA per cell, two per SM, on the SMs left
  // free by the clusters (at least one SM's worth; later CTAs find the queue
  // drained)
  int grid_s = 0;
  if (split) {
    int per_sm_s = 0;
    MSFEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_s, Ls->fn, Ls->nt, Ls->smem));
    if (per_sm_s < 1) return fail(MSFEM_ERR_UNSUPPORTED, "kernel does not fit on an SM");
    per_sm_s = std::min(per_sm_s, Ls->minb);
    const int free_sms = std::max(1, h->sm_count - ncl * L.cluster);
    grid_s = std::max(1, std::min(nc - n_large, free_sms * per_sm_s));
  }
  unsigned char *work = nullptr, *work_s = nullptr;
  size_t slot_bytes = L.slot_bytes;
  if (slot_bytes) {
    MSFEM_CUDA(h->work.ensure(slot_bytes * (slots + grid_s)));
    work = h->work.as<unsigned char>();
    work_s = work + slot_bytes * slots;
  }
  auto launch_basis = [&](void **args) -> cudaError_t {
    if (L.cluster > 1) return cudaLaunchKernelExC(&ccfg, L.fn, args);
    return cudaLaunchKernel(L.fn, dim3(grid), dim3(L.nt), args, L.smem, h->stream);
  };
  // the whole launch sequence on h->stream (the small cells forked to the
  // side stream and joined back)
  auto launch_all = [&]() -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(p.queue, 0, 2 * sizeof(unsigned int), h->stream);
    if (e != cudaSuccess || nc == 0) return e;
    if (split) {
      if ((e = cudaEventRecord(h->ev_fork, h->stream)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(h->side_stream, h->ev_fork, 0)) != cudaSuccess) return e;
    }
    void *args2[] = {&p};
    void *args3[] = {&p, &work, &slot_bytes};
    if ((e = launch_basis(slot_bytes ? args3 : args2)) != cudaSuccess) return e;
    if (split) {
      void *args_s[] = {&ps, &work_s, &slot_bytes};
      if ((e = cudaLaunchKernel(Ls->fn, dim3(grid_s), dim3(Ls->nt), args_s, Ls->smem, h->side_stream)) !=
          cudaSuccess)
        return e;
      if ((e = cudaEventRecord(h->ev_join, h->side_stream)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(h->stream, h->ev_join, 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  // Device-resident asynchronous calls replay a CUDA graph of the
  // queue-reset + basis-kernel sequence; it is re-captured whenever the
  // launch parameters (pointers, sizes, tuning) change.
  const bool graph_ok = dev && !stats && nc > 0 && h->use_graphs && h->stream != nullptr &&
                        h->stream != cudaStreamLegacy && h->stream != cudaStreamPerThread;
  MSFEM_CUDA(cudaEventRecord(h->ev0, h->stream));
  if (graph_ok) {
    std::string key(reinterpret_cast<const char *>(&p), sizeof(p));
    key.append(reinterpret_cast<const char *>(&L.fn), sizeof(L.fn));
    key.append(reinterpret_cast<const char *>(&L.nt), sizeof(L.nt));
    key.append(reinterpret_cast<const char *>(&L.smem), sizeof(L.smem));
    key.append(reinterpret_cast<const char *>(&slot_bytes), sizeof(slot_bytes));
    key.append(reinterpret_cast<const char *>(&grid), sizeof(grid));
    key.append(reinterpret_cast<const char *>(&work), sizeof(work));
    key.append(reinterpret_cast<const char *>(&h->stream), sizeof(h->stream));
    key.append(reinterpret_cast<const char *>(&split), sizeof(split));
    if (split) {
      key.append(reinterpret_cast<const char *>(&ps), sizeof(ps));
      key.append(reinterpret_cast<const char *>(&Ls->fn), sizeof(Ls->fn));
      key.append(reinterpret_cast<const char *>(&grid_s), sizeof(grid_s));
    }
    if (key != h->graph_key || !h->graph_exec) {
      if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
      h->graph_exec = nullptr;
      h->graph_key.clear();
      cudaGraph_t graph = nullptr;
      MSFEM_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      const cudaError_t e1 = launch_all();
      const cudaError_t e3 = cudaStreamEndCapture(h->stream, &graph);
      if (e1 != cudaSuccess || e3 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(MSFEM_ERR_CUDA, std::string("graph capture failed: ") +
                                        cudaGetErrorString(e1 != cudaSuccess ? e1 : e3));
      }
      const cudaError_t e4 = cudaGraphInstantiate(&h->graph_exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e4 != cudaSuccess) {
        h->graph_exec = nullptr;
        return fail(MSFEM_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e4));
      }
      h->graph_key = key;
      h->graph_captures++;
    }
    MSFEM_CUDA(cudaGraphLaunch(h->graph_exec, h->stream));
    launches += split ? 2 : 1;
    h->graph_launches++;
  } else {
    MSFEM_CUDA(launch_all());
    if (nc > 0) launches += split ? 2 : 1;
  }
  MSFEM_CUDA(cudaEventRecord(h->ev1, h->stream));

  // ---- results
  std::vector<int32_t> st_h, it_h, rf_h;
  std::vector<double> rr_h;
  const bool need_host = !dev || stats;
  if (!dev) {
    if (nc > 0) {
      MSFEM_CUDA(cudaMemcpyAsync(M, p.M, sizeof(double) * nc * nv * nv, cudaMemcpyDeviceToHost, h->stream));
      MSFEM_CUDA(cudaMemcpyAsync(F, p.F, sizeof(double) * nc * nv, cudaMemcpyDeviceToHost, h->stream));
      d2h += sizeof(double) * (int64_t)nc * (nv * nv + nv);
      if (basis) {
        MSFEM_CUDA(cudaMemcpyAsync(basis, p.basis, sizeof(double) * basis_total, cudaMemcpyDeviceToHost, h->stream));
        d2h += sizeof(double) * basis_total;
      }
      if (cell_status) {
        MSFEM_CUDA(cudaMemcpyAsync(cell_status, p.status, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost, h->stream));
        d2h += sizeof(int32_t) * nc;
      }
      if (iterations) {
        MSFEM_CUDA(cudaMemcpyAsync(iterations, p.iters, sizeof(int32_t) * nc * nv, cudaMemcpyDeviceToHost, h->stream));
        d2h += sizeof(int32_t) * nc * nv;
      }
    }
  }
  int nfail = 0;
  if (need_host && nc > 0) {
    st_h.resize(nc);
    it_h.resize((size_t)nc * nv);
    rr_h.resize(nc);
    rf_h.resize(nc);
    MSFEM_CUDA(cudaMemcpyAsync(st_h.data(), p.status, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost, h->stream));
    MSFEM_CUDA(cudaMemcpyAsync(it_h.data(), p.iters, sizeof(int32_t) * nc * nv, cudaMemcpyDeviceToHost, h->stream));
    MSFEM_CUDA(cudaMemcpyAsync(rr_h.data(), p.rel_res, sizeof(double) * nc, cudaMemcpyDeviceToHost, h->stream));
    MSFEM_CUDA(cudaMemcpyAsync(rf_h.data(), p.refinements, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost, h->stream));
  }
  if (need_host) MSFEM_CUDA(cudaStreamSynchronize(h->stream));
  if (need_host && d->warm_start == MSFEM_WARM_SURROGATE && nc > 0 && (rc = surrogate_check(h->surrogate)))
    return rc;
  for (int c = 0; c < (int)st_h.size(); ++c) nfail += st_h[c] != MSFEM_CELL_CONVERGED;
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->solves = (int64_t)nc * nv;
    stats->cells_failed = nfail;
    stats->cells_converged = nc - nfail;
    int64_t tot = 0;
    int itmax = 0, rfmax = 0;
    double rmax = 0.0;
    for (size_t i = 0; i < it_h.size(); ++i) { tot += it_h[i]; itmax = std::max(itmax, it_h[i]); }
    for (int c = 0; c < (int)rr_h.size(); ++c) {
      if (!(rr_h[c] <= rmax)) rmax = rr_h[c];  // NaN propagates
      rfmax = std::max(rfmax, rf_h[c]);
    }
    stats->iterations_total = tot;
    stats->iterations_max = itmax;
    stats->refinements_max = rfmax;
    stats->max_rel_residual = rmax;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev0, h->ev1) == cudaSuccess) stats->kernel_ms = ms;
    stats->kernel_launches = launches;
    stats->ctas_per_sm = per_sm;
    stats->h2d_bytes = h2d;
    stats->d2h_bytes = d2h;
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  }
  if (nfail) return fail(MSFEM_ERR_NOT_CONVERGED, std::to_string(nfail) + " cell(s) failed; see cell_status");
  return MSFEM_OK;
}

void fill_tuning(const Tune &t, int dim, int nmax, int precision, msfem_tuning *out) {
  const std::vector<Launch> c = candidates(dim, nmax, precision == MSFEM_PREC_MIXED);
  std::memset(out, 0, sizeof(*out));
  out->dim = dim;
  out->n_max = nmax;
  out->precision = precision;
  out->variant = t.variant;
  out->n_variants = (int)c.size();
  if (t.variant >= 0 && t.variant < (int)c.size()) {
    out->threads = c[t.variant].nt;
    out->rows_per_thread = c[t.variant].rows;
    out->ctas_per_sm = c[t.variant].minb;
    out->poly_degree = c[t.variant].poly;
    out->cluster_ctas = c[t.variant].cluster;
    out->coarse_spacing = c[t.variant].coarse;
  }
  out->cheb_ratio = t.cheb_ratio;
  out->check_interval = t.check_interval;
  out->inner_tol = t.inner_tol;
  out->ms_per_solve = t.ms_per_solve;
}

}  // namespace

extern "C" {

int msfem_run_batch(msfem_handle *h, const msfem_batch_desc *d, double *M, double *F,
                    double *basis, int32_t *cell_status, int32_t *iterations,
                    msfem_stats *stats) {
  return run_batch_impl(h, d, M, F, basis, cell_status, iterations, stats, nullptr);
}

int msfem_energy_error(msfem_handle *h, const msfem_batch_desc *d, const double *basis,
                       const double *basis_ref, double *err, double *ref_norm) {
  if (!h) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  int rc = validate(d);
  if (rc) return rc;
  if (d->n_cells > 0 && (!basis || !basis_ref || !err || !ref_norm))
    return fail(MSFEM_ERR_INVALID_ARG, "basis, basis_ref, err and ref_norm are required");
  if (d->n_cells == 0) return MSFEM_OK;
  MSFEM_CUDA(cudaSetDevice(h->device));
  const int nv = 1 << d->dim, nc = d->n_cells;
  const bool dev = d->memory == MSFEM_MEM_DEVICE;
  std::vector<int32_t> nf;
  if ((rc = host_nfine(h, d, nf))) return rc;
  msfem_batch_desc dd = *d;
  dd.warm_start = MSFEM_WARM_NONE;  // the network is not involved
  KernelParams p{};
  int64_t basis_total = 0, h2d = 0;
  int launches = 0;
  if ((rc = prepare_inputs(h, &dd, nf, p, basis_total, h2d, launches))) return rc;
  const double *a = nullptr, *r = nullptr;
  if ((rc = upload<double>(h, h->basis, basis, (size_t)basis_total, dev, &a, &h2d))) return rc;
  if ((rc = upload<double>(h, h->warm, basis_ref, (size_t)basis_total, dev, &r, &h2d))) return rc;
  double *e = err, *n = ref_norm;
  if (!dev) {
    MSFEM_CUDA(h->M.ensure(sizeof(double) * nc * nv));
    MSFEM_CUDA(h->F.ensure(sizeof(double) * nc * nv));
    e = h->M.as<double>();
    n = h->F.as<double>();
  }
  const int grid = std::max(1, std::min(nc, 4 * h->sm_count));
  if (d->dim == 2)
    MSFEM_CUDA(msfem::launch_energy_2d(grid, h->stream, p, a, r, e, n));
  else
    MSFEM_CUDA(msfem::launch_energy_3d(grid, h->stream, p, a, r, e, n));
  if (!dev) {
    MSFEM_CUDA(cudaMemcpyAsync(err, e, sizeof(double) * nc * nv, cudaMemcpyDeviceToHost, h->stream));
    MSFEM_CUDA(cudaMemcpyAsync(ref_norm, n, sizeof(double) * nc * nv, cudaMemcpyDeviceToHost, h->stream));
    MSFEM_CUDA(cudaStreamSynchronize(h->stream));
  }
  return MSFEM_OK;
}

int msfem_reconstruct(msfem_handle *h, const msfem_batch_desc *d, const double *basis, const double *weights,
                      double *u) {
  if (!h) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  int rc = validate(d);
  if (rc) return rc;
  if (d->n_cells > 0 && (!basis || !weights || !u))
    return fail(MSFEM_ERR_INVALID_ARG, "basis, weights and u are required");
  if (d->n_cells == 0) return MSFEM_OK;
  MSFEM_CUDA(cudaSetDevice(h->device));
  const int dim = d->dim, nv = 1 << dim, nc = d->n_cells;
  const bool dev = d->memory == MSFEM_MEM_DEVICE;
  std::vector<int32_t> nf;
  if ((rc = host_nfine(h, d, nf))) return rc;
  int64_t h2d = 0, basis_total = (int64_t)nc * nv * ipow(d->n_fine + 1, dim);
  const int32_t *nfd = nullptr;
  const int64_t *boffd = nullptr;
  if (d->n_fine_per_cell) {
    std::vector<int64_t> boff(nc);
    basis_total = 0;
    for (int c = 0; c < nc; ++c) {
      boff[c] = basis_total;
      basis_total += (int64_t)nv * ipow(nf[c] + 1, dim);
    }
    if ((rc = upload<int32_t>(h, h->nfine, d->n_fine_per_cell, (size_t)nc, dev, &nfd, &h2d))) return rc;
    if ((rc = upload<int64_t>(h, h->boff, boff.data(), boff.size(), false, &boffd, &h2d))) return rc;
  }
  const double *b = nullptr, *w = nullptr;
  if ((rc = upload<double>(h, h->basis, basis, (size_t)basis_total, dev, &b, &h2d))) return rc;
  if ((rc = upload<double>(h, h->F, weights, (size_t)nc * nv, dev, &w, &h2d))) return rc;
  const int64_t u_total = basis_total / nv;
  double *ud = u;
  if (!dev) {
    MSFEM_CUDA(h->warm.ensure(sizeof(double) * (size_t)u_total));
    ud = h->warm.as<double>();
  }
  const int grid = std::max(1, std::min(nc, 8 * h->sm_count));
  msfem::reconstruct_kernel<<<grid, 256, 0, h->stream>>>(dim, nc, d->n_fine, nfd, boffd, b, w, ud);
  MSFEM_CUDA(cudaGetLastError());
  if (!dev) {
    MSFEM_CUDA(cudaMemcpyAsync(u, ud, sizeof(double) * (size_t)u_total, cudaMemcpyDeviceToHost, h->stream));
    MSFEM_CUDA(cudaStreamSynchronize(h->stream));
  }
  return MSFEM_OK;
}

int msfem_set_tuning(msfem_handle *h, const msfem_tuning *t) {
  if (!h || !t) return fail(MSFEM_ERR_INVALID_ARG, "handle and tuning are required");
  if (t->dim != 2 && t->dim != 3) return fail(MSFEM_ERR_INVALID_ARG, "tuning dim must be 2 or 3");
  const bool mixed = t->precision == MSFEM_PREC_MIXED;
  const std::vector<Launch> c = candidates(t->dim, t->n_max, mixed);
  if (t->variant < 0 || t->variant >= (int)c.size())
    return fail(MSFEM_ERR_INVALID_ARG, "tuning variant out of range");
  if (t->check_interval < 0 || !(t->inner_tol > 0.0f && t->inner_tol < 1.0f))
    return fail(MSFEM_ERR_INVALID_ARG, "tuning parameters out of range");
  Tune tn;
  tn.variant = t->variant;
  tn.check_interval = t->check_interval;
  tn.inner_tol = t->inner_tol;
  tn.cheb_ratio = t->cheb_ratio > 1.0f ? t->cheb_ratio : Tune().cheb_ratio;
  tn.ms_per_solve = t->ms_per_solve;
  h->tuning[tune_key(t->dim, t->n_max, mixed)] = tn;
  return MSFEM_OK;
}

int msfem_describe_tuning(msfem_tuning *t) {
  if (!t) return fail(MSFEM_ERR_INVALID_ARG, "tuning is required");
  if (t->dim != 2 && t->dim != 3) return fail(MSFEM_ERR_INVALID_ARG, "tuning dim must be 2 or 3");
  const bool mixed = t->precision == MSFEM_PREC_MIXED;
  const std::vector<Launch> c = candidates(t->dim, t->n_max, mixed);
  if (t->variant < 0 || t->variant >= (int)c.size())
    return fail(MSFEM_ERR_INVALID_ARG, "tuning variant out of range");
  const Launch &L = c[t->variant];
  t->n_variants = (int)c.size();
  t->threads = L.nt;
  t->rows_per_thread = L.rows;
  t->ctas_per_sm = L.minb;
  t->poly_degree = L.poly;
  t->cluster_ctas = L.cluster;
  t->coarse_spacing = L.coarse;
  return MSFEM_OK;
}

int msfem_autotune(msfem_handle *h, const msfem_batch_desc *d, int32_t sample_cells,
                   msfem_tuning *result) {
  if (!h) return fail(MSFEM_ERR_INVALID_ARG, "handle is NULL");
  int rc = validate(d);
  if (rc) return rc;
  if (d->n_cells < 1) return fail(MSFEM_ERR_INVALID_ARG, "autotune needs at least one cell");
  MSFEM_CUDA(cudaSetDevice(h->device));
  std::vector<int32_t> nf;
  if ((rc = host_nfine(h, d, nf))) return rc;
  int nmax = d->n_fine;
  if (d->n_fine_per_cell) nmax = *std::max_element(nf.begin(), nf.end());
  const bool mixed = d->precision == MSFEM_PREC_MIXED;
  const std::vector<Launch> cands = candidates(d->dim, nmax, mixed);
  if (cands.empty()) return fail(MSFEM_ERR_UNSUPPORTED, "no kernel for this size");
  // sample: a prefix of the cells (uniform N without caller offsets), else the batch
  msfem_batch_desc s = *d;
  if (!d->n_fine_per_cell && !d->coef.qp_offset && sample_cells > 0)
    s.n_cells = std::min(d->n_cells, sample_cells);
  if (d->warm_start == MSFEM_WARM_USER) s.warm_start = MSFEM_WARM_NONE;
  const int nv = 1 << d->dim, nc = s.n_cells;
  const bool dev = d->memory == MSFEM_MEM_DEVICE;
  std::vector<double> Mh, Fh;
  double *Mp = nullptr, *Fp = nullptr;
  if (dev) {
    MSFEM_CUDA(h->M.ensure(sizeof(double) * nc * nv * nv));
    MSFEM_CUDA(h->F.ensure(sizeof(double) * nc * nv));
    Mp = h->M.as<double>();
    Fp = h->F.as<double>();
  } else {
    Mh.resize((size_t)nc * nv * nv);
    Fh.resize((size_t)nc * nv);
    Mp = Mh.data();
    Fp = Fh.data();
  }
  std::vector<Tune> trials;
  for (int v = 0; v < (int)cands.size(); ++v) {
    if (mixed) {
      for (float it : {1e-4f, 1e-5f, 1e-6f, 1e-7f}) {
        if (cands[v].poly > 0) {
          // two-level shapes smooth with a narrower interval than the
          // polynomial preconditioner alone
          const std::vector<float> ratios = cands[v].coarse > 0 ? std::vector<float>{12.0f, 15.0f, 20.0f}
                                                                 : std::vector<float>{10.0f, 30.0f, 100.0f};
          for (float ratio : ratios) {
            Tune t;
            t.variant = v;
            t.inner_tol = it;
            t.cheb_ratio = ratio;
            trials.push_back(t);
          }
        } else {
          Tune t;
          t.variant = v;
          t.inner_tol = it;
          trials.push_back(t);
        }
      }
    } else {
      for (int ci : {0, 1, 4}) {
        Tune t;
        t.variant = v;
        t.check_interval = ci;
        trials.push_back(t);
      }
    }
  }
  Tune best;
  double best_ms = 1e300;
  for (Tune &t : trials) {
    msfem_stats st;
    double ms = 1e300;
    for (int rep = 0; rep < 2; ++rep) {
      rc = run_batch_impl(h, &s, Mp, Fp, nullptr, nullptr, nullptr, &st, &t);
      if (rc != MSFEM_OK && rc != MSFEM_ERR_NOT_CONVERGED) return rc;
      if (st.cells_failed == 0) ms = std::min(ms, st.kernel_ms);
    }
    t.ms_per_solve = ms / std::max<int64_t>(1, (int64_t)nc * nv);
    if (ms < best_ms) {
      best_ms = ms;
      best = t;
    }
  }
  if (best_ms >= 1e300) return fail(MSFEM_ERR_NOT_CONVERGED, "no launch choice converged on the sample");
  h->tuning[tune_key(d->dim, nmax, mixed)] = best;
  if (result) fill_tuning(best, d->dim, nmax, d->precision, result);
  return MSFEM_OK;
}

}  // extern "C"
