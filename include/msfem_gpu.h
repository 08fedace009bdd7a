/*
 * msfem_gpu.h -- C-ABI of libmsfem_gpu.so, the GB300 (sm_103a) engine for the
 * per-coarse-cell multiscale basis problems of an MsFEM discretisation of
 * -div(A(x) grad u) = f.
 *
 * For every coarse cell K (a quadrilateral / hexahedron given by its 2^d
 * corners in deal.II vertex order) the engine
 *   1. builds the local N^d fine Q1 mesh (uniform refinement of K),
 *   2. assembles the fine Q1 form  int_K grad(psi_i) . A(x) grad(psi_j)  with a
 *      2^d-point Gauss rule per fine cell, and the load  int_K f psi_i,
 *   3. solves the 2^d Dirichlet problems whose boundary data are the coarse
 *      Q1 nodal functions (value 1 at coarse vertex i, 0 at the others),
 *   4. integrates the coarse element matrix  M_ij = phi_i^T A phi_j  and the
 *      coarse load  F_i = phi_i^T b  from those multiscale basis functions.
 *
 * Reference interfaces replaced (konsim83/MPI-Parallel-Multiscale-Diffusion-FEM):
 *   msfem_run_batch      <- DiffusionProblemBasis<dim>::run()
 *                           include/base/diffusion_problem_basis.tpp:438-474
 *                           (make_grid :90-99, setup_system :102-156,
 *                            assemble_system :159-242, solve_iterative :293-317,
 *                            assemble_global_element_matrix :245-285)
 *                           called once per owned cell by
 *                           include/base/diffusion_problem_ms.tpp:81-87
 *   M output             <- get_global_element_matrix()  diffusion_problem_basis.tpp:320-325
 *   F output             <- get_global_element_rhs()     diffusion_problem_basis.tpp:328-333
 *   basis output         <- solution_vector[i], read by set_global_weights()
 *                           diffusion_problem_basis.tpp:352-377
 *   msfem_coef_desc      <- Coefficients::MatrixCoeff<dim>::value_list
 *                           include/coefficients/matrix_coeff.tpp:66-91,
 *                           Coefficients::RightHandSide<dim>::value_list
 *                           include/coefficients/right_hand_side.tpp:27-40
 *   Dirichlet data       <- Coefficients::BasisQ1<dim>  include/coefficients/basis_q1.tpp:26-158
 *   cell status / error  <- SolverControl::NoConvergence thrown by SolverCG
 *                           diffusion_problem_basis.tpp:297-306
 *
 * Conventions
 *   - All floating point input and output is IEEE FP64.
 *   - Coarse-cell corners: corners[cell][v][c], v in deal.II lexicographic
 *     vertex order (v = vx + 2 vy + 4 vz), c the coordinate.
 *   - Local fine nodes are numbered lexicographically, x fastest:
 *     node = ix + n (iy + n iz), n = N + 1.  (deal.II's own numbering is the
 *     cell-traversal order; callers that need it permute by support point.)
 *   - M[cell][i][j] is row-major with row i = test function, column j = trial,
 *     exactly as global_element_matrix(i_test, i_trial).
 *   - No pointer is retained after a call returns.  No C++ exception crosses
 *     this boundary; every entry point returns an msfem_status_code.
 *   - A handle is bound to one device and must not be used by two host
 *     threads at the same time.  One MPI rank = one handle = one GPU.
 */
#ifndef MSFEM_GPU_H_
#define MSFEM_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSFEM_ABI_VERSION 2

/* Largest supported local refinement per coarse cell. */
#define MSFEM_MAX_N_2D 32
#define MSFEM_MAX_N_3D 24

typedef enum msfem_status_code {
  MSFEM_OK = 0,
  MSFEM_ERR_INVALID_ARG = -1,   /* malformed descriptor / size out of range */
  MSFEM_ERR_CUDA = -2,          /* CUDA runtime error, see msfem_last_error */
  MSFEM_ERR_NO_DEVICE = -3,     /* no usable sm_103 device */
  MSFEM_ERR_UNSUPPORTED = -4,   /* combination not implemented */
  MSFEM_ERR_OUT_OF_MEMORY = -5,
  MSFEM_ERR_NOT_CONVERGED = -6  /* at least one cell did not reach tol: see cell_status */
} msfem_status_code;

/* Per-cell status word (cell_status output). */
typedef enum msfem_cell_status {
  MSFEM_CELL_CONVERGED = 0,
  MSFEM_CELL_MAXIT = 1,         /* maxit reached (reference: SolverControl::NoConvergence) */
  MSFEM_CELL_NAN = 2,           /* non-finite value met (bad coefficient, breakdown) */
  MSFEM_CELL_BAD_INPUT = 3      /* e.g. degenerate / inverted cell geometry */
} msfem_cell_status;

/* Coefficient A(x) kinds.  Scalar kinds mean A = a(x) I. */
typedef enum msfem_coef_kind {
  /* A = const symmetric tensor; params = (a11,a12,a22) in 2D,
   * (a11,a12,a13,a22,a23,a33) in 3D. */
  MSFEM_COEF_CONSTANT = 0,
  /* The reference's own Coefficients::MatrixCoeff<dim> (matrix_coeff.tpp:17-91):
   * c(x) = 1 - 0.9999 (0.5 sin(2 PI_D 57 x) + 0.5 sin(2 PI_D 57 y)),
   * A = R diag(c) R^T, PI_D = 3.14592653509793218403 as in coefficients.h:21,
   * R the rotation by PI_D/3 (2D) or the ZXZ Euler matrix (PI_D/3, PI_D/6, PI_D/4) (3D). */
  MSFEM_COEF_REFERENCE = 1,
  /* a = 1 + amp sin(2 pi x/eps) sin(2 pi y/eps) [sin(2 pi z/eps) in 3D];
   * params = (amp, eps). */
  MSFEM_COEF_SINSIN = 2,
  /* Random Fourier fields g_f(x) = sum_m amp_m cos(k_m . x + phase_m), table
   * modes[f][m][5] = (kx, ky, kz, amp, phase).  2D: 3 fields (g1, g2, theta),
   * A = R(theta) diag(exp g1, exp g2) R(theta)^T.  3D: 1 field, a = exp g1. */
  MSFEM_COEF_FOURIER = 3,
  /* a = 1 + (params[0] - 1) * [x inside any sphere]; spheres[s] = (cx,cy,cz,r)
   * (2D: discs, cz ignored). */
  MSFEM_COEF_SPHERES = 4,
  /* Values at the Gauss points, caller-tabulated (generic path for any
   * TensorFunction: tabulate with value_list and pass the values).  Per cell a
   * block of ncomp * 2^d * N^d doubles, ordered [comp][q][fine cell], fine
   * cells lexicographic (x fastest), q the deal.II QGauss(2) point order
   * (x fastest).  ncomp = 1 (scalar) or d(d+1)/2 (symmetric tensor, component
   * order as for CONSTANT). */
  MSFEM_COEF_TABULATED = 5
} msfem_coef_kind;

typedef enum msfem_precision {
  MSFEM_PREC_FP64 = 0,          /* plain FP64 Jacobi-PCG (the drop-in form) */
  MSFEM_PREC_MIXED = 1          /* FP32 inner PCG + FP64 residual refinement */
} msfem_precision;

typedef enum msfem_memory {
  MSFEM_MEM_HOST = 0,           /* all descriptor/output pointers are host memory; inputs of
                                   1 MB or more in pinned (device-mapped) memory are read in
                                   place by the kernels, pageable ones are copied */
  MSFEM_MEM_DEVICE = 1          /* all descriptor/output pointers are device memory */
} msfem_memory;

typedef enum msfem_warm_start {
  MSFEM_WARM_NONE = 0,          /* x0 = 0 in the interior (reference behaviour) */
  MSFEM_WARM_USER = 1,          /* x0 = warm_basis (interior values used) */
  MSFEM_WARM_SURROGATE = 2      /* x0 = prediction of the surrogate attached to the handle */
} msfem_warm_start;

typedef struct msfem_coef_desc {
  int32_t kind;                 /* msfem_coef_kind */
  int32_t ncomp;                /* TABULATED only */
  double params[8];
  const double *qp_values;      /* TABULATED */
  const int64_t *qp_offset;     /* TABULATED, per-cell offset in doubles; NULL = packed cell
                                   blocks of ncomp 2^d N_c^d doubles in cell order */
  const double *modes;          /* FOURIER [n_fields][n_modes][5] */
  int32_t n_modes;
  int32_t n_spheres;
  const double *spheres;        /* SPHERES [n_spheres][4], always host memory */
} msfem_coef_desc;

typedef struct msfem_batch_desc {
  int32_t dim;                  /* 2 or 3 */
  int32_t n_cells;
  int32_t n_fine;               /* N for all cells when n_fine_per_cell == NULL */
  int32_t precision;            /* msfem_precision */
  const double *corners;        /* [n_cells][2^dim][dim] */
  const int32_t *n_fine_per_cell; /* optional, [n_cells] (uneven local refinement) */
  msfem_coef_desc coef;
  double f_value;               /* constant right-hand side f (reference: 2.0); see f_qp_values */
  double tol;                   /* l2 residual tolerance, relative or absolute (tol_absolute) */
  int32_t maxit;                /* CG iteration cap per solve (reference: 1000) */
  int32_t memory;               /* msfem_memory */
  int32_t warm_start;           /* msfem_warm_start */
  int32_t check_interval;       /* residual-norm check every k iterations, 0 = tuned default */
  const double *warm_basis;     /* [n_cells][2^dim][n^dim], WARM_USER only; uneven N: cell blocks of 2^d (N_c+1)^d */
  /* Stopping rule of every solve.  0: relative, ||b - A x|| <= tol ||b||.
   * 1: absolute, ||b - A x|| <= tol, the reference's SolverControl(1000, 1e-12)
   * (diffusion_problem_basis.tpp:297, deal.II SolverCG checks the l2 norm of
   * the unpreconditioned residual, from step 0).  The residual is that of the
   * interior rows of the unscaled fine Q1 system with the Dirichlet lifting. */
  int32_t tol_absolute;
  int32_t reserved0;            /* must be 0 */
  /* Optional right-hand side f at the Gauss points, replacing f_value:
   * RightHandSide<dim>::value_list at the QGauss(2) points of every fine cell
   * (diffusion_problem_basis.tpp:204-205, :219-220; right_hand_side.tpp:27-40).
   * Per cell a block of 2^d N^d doubles ordered [q][fine cell] (the scalar
   * TABULATED layout); f_qp_offset[cell] = start of the cell's block in
   * doubles, NULL = packed blocks in cell order.  f only enters the coarse
   * load F (the local problems have a zero right-hand side, :455). */
  const double *f_qp_values;
  const int64_t *f_qp_offset;
} msfem_batch_desc;

typedef struct msfem_stats {
  int64_t solves;               /* 2^d * n_cells */
  int64_t cells_converged;
  int64_t cells_failed;
  int64_t iterations_total;     /* CG iterations summed over solves (inner FP32 ones in MIXED) */
  int32_t iterations_max;
  int32_t refinements_max;      /* MIXED: outer FP64 refinement steps, max over cells */
  double max_rel_residual;      /* true FP64 ||b - A phi||/||b||, max over solves */
  double kernel_ms;             /* device time of the solve kernel(s) */
  double total_ms;              /* wall time of the call */
  int32_t kernel_launches;      /* kernels this call launched */
  int32_t ctas_per_sm;
  int64_t h2d_bytes;
  int64_t d2h_bytes;
} msfem_stats;

typedef struct msfem_handle msfem_handle;

/* Create a handle on CUDA device `device`.  Fails with MSFEM_ERR_NO_DEVICE
 * when the device is absent or not an sm_103 part. */
int msfem_create(msfem_handle **handle, int device);

/* Release all device buffers, streams and graphs of the handle. */
int msfem_destroy(msfem_handle *handle);

/* Launch on this stream (a cudaStream_t) instead of the handle's own.  NULL
 * restores the handle's own stream; to launch on the legacy default stream
 * pass cudaStreamLegacy. */
int msfem_set_stream(msfem_handle *handle, void *cuda_stream);

/* CUDA-graph use of the handle: how many graphs msfem_run_batch has captured
 * and how many graph launches it has made.  Device-resident calls without
 * stats (desc->memory == MSFEM_MEM_DEVICE, stats == NULL) on a stream other
 * than the legacy default stream replay one graph of the queue reset and the
 * basis kernel; a change of pointers, sizes or tuning re-captures it.  No
 * counterpart in the reference (diagnostics of the batching layer). */
int msfem_graph_info(msfem_handle *handle, int64_t *captures, int64_t *replays);

/* Compute the multiscale basis of a batch of coarse cells.
 *   M            [n_cells][2^d][2^d]   coarse element matrices
 *   F            [n_cells][2^d]        coarse element loads
 *   basis        [n_cells][2^d][n^d]   optional (NULL): basis values at the fine
 *                nodes (uneven N: cell blocks of 2^d (N_c+1)^d, in cell order)
 *   cell_status  [n_cells]             optional, msfem_cell_status
 *   iterations   [n_cells][2^d]        optional, CG iterations per solve
 *   stats        optional
 * Output pointers follow desc->memory.  Returns MSFEM_ERR_NOT_CONVERGED when
 * some cell failed (its status says why); outputs of the other cells are valid. */
int msfem_run_batch(msfem_handle *handle, const msfem_batch_desc *desc,
                    double *M, double *F, double *basis,
                    int32_t *cell_status, int32_t *iterations,
                    msfem_stats *stats);

/* Energy-norm error of every basis function against a reference basis:
 *   err      [n_cells][2^d]   ||phi_i - ref_i||_A
 *   ref_norm [n_cells][2^d]   ||ref_i||_A   (= sqrt(M_ii) for a converged ref)
 * with A the cell's fine Q1 stiffness matrix over all nodes, the
 * unconstrained diffusion_matrix of diffusion_problem_basis.tpp:159-242
 * assembled from desc's cells and coefficient, summed element by element.
 * basis and basis_ref use msfem_run_batch's basis layout.  All four arrays
 * follow desc->memory; DEVICE calls are asynchronous on the handle's stream.
 * A malformed cell gets NaN.  No counterpart in the reference (it reports no
 * basis errors); it serves the error report of the mixed and warm-started
 * forms against an FP64 solve at a tighter tolerance. */
int msfem_energy_error(msfem_handle *handle, const msfem_batch_desc *desc,
                       const double *basis, const double *basis_ref,
                       double *err, double *ref_norm);

/* Fine-scale solution in every cell from its multiscale basis and the
 * coarse solution: u[cell][node] = sum_i w[cell][i] phi_i[cell][node].
 * Replaces set_global_weights + the per-cell reconstruction of the fine
 * solution (diffusion_problem_basis.tpp:352-377, used by
 * diffusion_problem_ms.tpp:299-325 for output).
 *   basis    msfem_run_batch's basis layout ([cell][2^d][(N+1)^d]; uneven N:
 *            cell blocks of 2^d (N_c+1)^d)
 *   weights  [n_cells][2^d], the coarse solution at the cell's vertices in
 *            the order of M/F
 *   u        [cell][(N+1)^d] lexicographic fine nodes (uneven N: cell blocks
 *            of (N_c+1)^d)
 * desc supplies dim, n_cells, N (uniform or per cell) and the memory mode;
 * its coefficient is not used.  DEVICE calls are asynchronous on the
 * handle's stream. */
int msfem_reconstruct(msfem_handle *handle, const msfem_batch_desc *desc, const double *basis,
                      const double *weights, double *u);

/* Evaluate the coefficient of desc->coef (any analytic kind) at the Gauss
 * points of every fine cell of the batch, in the TABULATED layout, on the
 * device.  qp_values is a device pointer when desc->memory is DEVICE. */
int msfem_tabulate_coefficient(msfem_handle *handle,
                               const msfem_batch_desc *desc,
                               int32_t ncomp, double *qp_values);

/* Launch choice for one (dim, N class, precision): which compiled CTA shape
 * (threads, strip height, CTAs per SM) the batch kernel uses, the FP64
 * form's residual-check interval and the mixed form's inner FP32 reduction.
 * No counterpart in the reference (its solver has no launch parameters). */
typedef struct msfem_tuning {
  int32_t dim;              /* key */
  int32_t n_max;            /* key: largest N of the batch (selects the N class) */
  int32_t precision;        /* key: msfem_precision */
  int32_t variant;          /* index of the compiled CTA shape */
  int32_t threads;          /* output: CTA size of that shape */
  int32_t rows_per_thread;  /* output: strip height (mixed kernels) */
  int32_t ctas_per_sm;      /* output: occupancy the shape is compiled for */
  int32_t check_interval;   /* FP64: residual-norm check interval, 0 = adaptive */
  float inner_tol;          /* MIXED: inner FP32 CG relative reduction */
  int32_t n_variants;       /* output: compiled shapes for this key */
  double ms_per_solve;      /* output of msfem_autotune: device time per basis solve */
  float cheb_ratio;         /* MIXED, polynomial-preconditioned shapes: b / a of the
                               Chebyshev interval [a, b], b the Gershgorin bound */
  int32_t poly_degree;      /* output: degree of that shape's polynomial preconditioner
                               (0 = Jacobi-scaled CG) */
  int32_t cluster_ctas;     /* output: CTAs of a thread-block cluster sharing one cell
                               (3D cluster shapes), 1 = one CTA per cell */
  int32_t coarse_spacing;   /* output: fine cells per coarse-grid interval of that shape's
                               two-level inner preconditioner (MIXED 2D), 0 = none */
} msfem_tuning;

/* Time every compiled shape and parameter choice for desc's key on a prefix
 * of at most sample_cells cells (the whole batch for uneven N), keep the
 * fastest in the handle (used by later msfem_run_batch calls with the same
 * key) and report it in result (nullable). */
int msfem_autotune(msfem_handle *handle, const msfem_batch_desc *desc,
                   int32_t sample_cells, msfem_tuning *result);

/* Install a launch choice (e.g. one saved from an earlier msfem_autotune). */
int msfem_set_tuning(msfem_handle *handle, const msfem_tuning *tuning);

/* Describe a compiled launch shape without running anything: for the key
 * (dim, n_max, precision) and variant of *tuning, fill the output fields
 * threads, rows_per_thread, ctas_per_sm, n_variants, poly_degree,
 * cluster_ctas and coarse_spacing; the other fields are left as given.
 * MSFEM_ERR_INVALID_ARG for an unknown key or a variant out of range. */
int msfem_describe_tuning(msfem_tuning *tuning);

/* Number of doubles msfem_tabulate_coefficient writes for this batch. */
int64_t msfem_tabulated_size(const msfem_batch_desc *desc, int32_t ncomp);

/* Largest batch msfem_run_batch_noalloc accepts (its fixed scratch holds a
 * work-queue counter plus 12 bytes per cell: about 0.75 MB per device). */
#define MSFEM_NOALLOC_MAX_CELLS 65536

/* No counterpart in the reference: an entry point for callers that cannot
 * allocate device memory.  msfem_run_batch sizes its device buffers on demand
 * (cudaMalloc on the first call, and again whenever a batch outgrows them).
 * Some callers cannot allow that: a framework that owns every device
 * allocation of the process (a fixed memory budget or pool, where a hidden
 * cudaMalloc either fails or breaks the accounting), or a latency-critical
 * time loop, where cudaMalloc/cudaFree synchronise the whole device.
 *
 * This variant of the 2D basis kernel allocates nothing: no cudaMalloc, no
 * cudaFree, no handle, no allocating library call.  Its scratch (the
 * work-queue counter and per-cell residual / refinement words) is one
 * file-scope device array of fixed size in libmsfem_gpu.so, which every GPU
 * that loads the library holds until the process exits.
 *   - 2D only, uniform N (n_fine_per_cell must be NULL), desc->memory must be
 *     MSFEM_MEM_DEVICE: every pointer in desc and every output is a device
 *     pointer the caller owns.  Coefficient kinds CONSTANT, REFERENCE, SINSIN
 *     and TABULATED (FOURIER/SPHERES need a tabulation buffer: tabulate first).
 *     Warm starts NONE and USER; MSFEM_WARM_SURROGATE is rejected
 *     (MSFEM_ERR_UNSUPPORTED): the network lives in a handle.
 *   - n_cells above MSFEM_NOALLOC_MAX_CELLS is rejected (MSFEM_ERR_INVALID_ARG).
 *   - It always runs the default compiled launch shape with the default
 *     parameters (residual-check interval, inner FP32 reduction): there is no
 *     handle, so msfem_autotune / msfem_set_tuning choices do not apply.
 *   - The first call on a device looks up the scratch array's device address
 *     (with that device current).
 *   - The call only enqueues work on `stream` (a cudaStream_t, NULL = legacy
 *     default stream) and returns; outputs are valid once the stream has
 *     completed, and per-cell failures are reported in cell_status only.
 *   - All calls share the one scratch array, which keeps the last call's
 *     contents; the counter is cleared on `stream` before each launch.  Calls
 *     that may overlap on the GPU (different streams without ordering) race on
 *     it: serialise them.
 * Results equal msfem_run_batch's on the same inputs with the default launch
 * choice. */
int msfem_run_batch_noalloc(const msfem_batch_desc *desc, double *M, double *F,
                            double *basis, int32_t *cell_status,
                            int32_t *iterations, void *stream);

/* ---------------------------------------------------------------------------
 * Learned warm start (no counterpart in the reference): a 6-layer 3x3
 * convolutional network, 3 -> 32 -> 32 -> 32 -> 32 -> 32 -> 4 channels, that
 * maps a 2D cell's coefficient on its 33 x 33 fine nodal grid (N = 32) to the
 * corrections delta_i = phi_i - Q1_i of the four basis functions.  BF16
 * weights and activations with FP32 accumulation on the tensor cores, FP32
 * master weights, Adam.  The CG always runs to the requested tolerance from
 * the predicted start, so the network only changes the iteration count.
 *   features  [n][3][33][33] FP32: log a11, a12/sqrt(a11 a22), log a22 at the nodes
 *   targets / predictions [n][4][33][33] FP32 (delta_i, zero on the boundary)
 *   parameters: FP32, per layer W [Cout][Cin][3][3] then b [Cout]
 * All feature / target / prediction pointers are device pointers.
 * ------------------------------------------------------------------------- */
typedef struct msfem_surrogate msfem_surrogate;

int64_t msfem_surrogate_param_count(void);

/* New network on the handle's device and stream, seeded uniform init. */
int msfem_surrogate_create(msfem_handle *handle, uint64_t seed, msfem_surrogate **net);
int msfem_surrogate_destroy(msfem_surrogate *net);
int msfem_surrogate_set_params(msfem_surrogate *net, const float *params_host);
int msfem_surrogate_get_params(msfem_surrogate *net, float *params_host);

/* Node features of a 2D, N = 32 batch whose coefficient is TABULATED in
 * device memory (desc->memory == MSFEM_MEM_DEVICE). */
int msfem_surrogate_features(msfem_handle *handle, const msfem_batch_desc *desc, float *features);

/* Training targets from computed basis functions: delta_i = phi_i - Q1_i at
 * the nodes, basis [n][4][33*33] FP64 -> delta [n][4][33][33] FP32. */
int msfem_surrogate_targets(msfem_handle *handle, const double *basis, int32_t n, float *delta);

/* Forward pass: predictions for n cells. */
int msfem_surrogate_predict(msfem_surrogate *net, const float *features, int32_t n, float *delta);

/* Loss (mean squared error over interior nodes) and parameter gradients
 * (host FP32, msfem_surrogate_param_count values) without updating. */
int msfem_surrogate_gradients(msfem_surrogate *net, const float *features, const float *targets,
                              int32_t batch, float *grads_host, double *loss);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on a batch. */
int msfem_surrogate_train_step(msfem_surrogate *net, const float *features, const float *targets,
                               int32_t batch, float lr, double *loss);

/* The network used by MSFEM_WARM_SURROGATE on this handle (NULL detaches). */
int msfem_attach_surrogate(msfem_handle *handle, msfem_surrogate *net);

/* Message of the last failing call on this thread. */
int msfem_last_error(char *buf, size_t len);

/* Library version string. */
const char *msfem_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MSFEM_GPU_H_ */
