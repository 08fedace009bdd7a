/*
 * msfem_oracle.h -- CPU FP64 restatement of the reference's local multiscale
 * basis computation.  TEST INFRASTRUCTURE ONLY: used by tests/, by the smoke
 * check and by bench.py's CPU baseline / reference arm, never by the product
 * library.
 *
 * Parity status: the reference (konsim83/MPI-Parallel-Multiscale-Diffusion-FEM)
 * cannot be built in this environment (deal.II, p4est, Trilinos and MPI are
 * absent) and its only test (test/test_dummy.cc) pins no numbers, so this
 * oracle is NOT pinned against reference outputs ("parity unpinned" at the
 * reference level).  It is pinned instead against analytic known answers
 * (constant diagonal tensors, where the multiscale basis is the Q1 basis and
 * the coarse matrix has a closed form) and structural invariants, and it is
 * cross-checked against an independent numpy restatement in tests/.
 *
 * Follows (file:line within the reference project):
 *   make_grid                      include/base/diffusion_problem_basis.tpp:90-99
 *   setup_system (constraints)     include/base/diffusion_problem_basis.tpp:102-156
 *   assemble_system                include/base/diffusion_problem_basis.tpp:159-242
 *   run() per-basis condense+solve include/base/diffusion_problem_basis.tpp:450-465
 *   solve_iterative (SSOR-CG)      include/base/diffusion_problem_basis.tpp:293-317
 *   assemble_global_element_matrix include/base/diffusion_problem_basis.tpp:245-285
 *   BasisQ1                        include/coefficients/basis_q1.tpp:26-158
 *   MatrixCoeff                    include/coefficients/matrix_coeff.tpp:17-91
 *   RightHandSide                  include/coefficients/right_hand_side.tpp:17-40
 *   PI_D                           include/coefficients/coefficients.h:21
 *   coarse MsFEM problem           include/base/diffusion_problem_ms.tpp:91-296
 *   DirichletBC / NeumannBC        include/coefficients/dirichlet_bc.tpp:17-43,
 *                                  include/coefficients/neumann_bc.tpp:17-41
 */
#ifndef MSFEM_ORACLE_H_
#define MSFEM_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Coefficient kinds: same numbering as msfem_coef_kind in include/msfem_gpu.h. */
enum { OC_COEF_CONSTANT = 0, OC_COEF_REFERENCE = 1, OC_COEF_SINSIN = 2,
       OC_COEF_FOURIER = 3, OC_COEF_SPHERES = 4, OC_COEF_TABULATED = 5 };

/* Local solvers. */
enum { OC_SOLVER_DIRECT = 0,      /* banded Cholesky of A_II: the FP64 oracle */
       OC_SOLVER_SSOR_CG = 1,     /* reference algorithm: SSOR(omega)-PCG on the condensed system */
       OC_SOLVER_JACOBI_CG = 2 }; /* the device algorithm: Jacobi-PCG, all 2^d RHS */

/* Orderings of the local unknowns (only SSOR depends on it). */
enum { OC_ORDER_LEX = 0, OC_ORDER_DEALII = 1 };

typedef struct oc_coef {
  int32_t kind;
  int32_t ncomp;
  double params[8];
  const double *qp_values;
  const int64_t *qp_offset;
  const double *modes;
  int32_t n_modes;
  int32_t n_spheres;
  const double *spheres;
} oc_coef;

typedef struct oc_batch {
  int32_t dim;
  int32_t n_cells;
  int32_t n_fine;
  int32_t solver;
  const double *corners;
  const int32_t *n_fine_per_cell;
  oc_coef coef;
  double f_value;
  double tol;             /* residual tolerance */
  int32_t tol_absolute;   /* 1: ||r|| <= tol (reference SolverControl), 0: ||r|| <= tol ||b|| */
  int32_t maxit;
  double omega;           /* SSOR relaxation, reference 1.6 */
  int32_t ordering;
  int32_t nthreads;
  int32_t raw_monomials;  /* 1: BasisQ1 from untranslated monomials exactly as basis_q1.tpp */
  /* optional right-hand side at the Gauss points (RightHandSide::value_list,
   * diffusion_problem_basis.tpp:204-205): per cell 2^d N^d values [q][fine
   * cell]; f_qp_offset NULL = packed blocks in cell order; NULL = f_value */
  const double *f_qp_values;
  const int64_t *f_qp_offset;
} oc_batch;

/* Whole batch.  M [n][2^d][2^d], F [n][2^d]; optional (may be NULL):
 * basis [cell blocks of 2^d (N_c+1)^d], iters [n][2^d], rel_res [n][2^d]
 * (true residual ||b - A_II u||/||b|| after the solve).  Returns the number
 * of solves that did not converge (0 = all converged), < 0 on bad input. */
int oc_run_batch(const oc_batch *b, double *M, double *F, double *basis,
                 int32_t *iters, double *rel_res);

/* Assembly of one cell: full (unconstrained) stencil st[n^d][3^d] and load
 * vector bl[n^d], exactly the matrix diffusion_matrix and vector global_rhs
 * of the reference (in lexicographic node order). */
int oc_assemble_cell(const oc_batch *b, int32_t cell, double *st, double *bl);

/* BasisQ1 Dirichlet data: values of the 2^d coarse Q1 nodal functions of
 * `cell` at point x (out[2^d]). */
void oc_basis_q1(const oc_batch *b, int32_t cell, const double *x, double *out);

/* Coefficient tensor A (row-major d x d) at point x; `cell`, `fc`, `q` locate
 * the Gauss point for the TABULATED kind. */
void oc_coef_eval(const oc_batch *b, int32_t cell, int32_t fc, int32_t q,
                  const double *x, double *A);

/* Tabulate the coefficient at all Gauss points in the TABULATED layout. */
int oc_tabulate(const oc_batch *b, int32_t ncomp, double *out);

/* Coarse MsFEM problem on [0,1]^d with K = 2^n_refine cells per direction
 * (coarse cell c = cx + K (cy + K cz)).  Assembles M/F, the Neumann face
 * terms and the Dirichlet data as diffusion_problem_ms.tpp:106-255 and
 * solves directly.  bc = 0: reference problem (DirichletBC on ids 0/2/4,
 * NeumannBC on ids 1/3/5); bc = 1: homogeneous Dirichlet on the whole
 * boundary.  u [(K+1)^d] lexicographic. */
int oc_coarse_solve(int32_t dim, int32_t K, const double *M, const double *F,
                    int32_t bc, double *u);

/* Corner coordinates of the K^d cells of the refined unit cube. */
void oc_unit_cube_corners(int32_t dim, int32_t K, double *corners);

#ifdef __cplusplus
}
#endif
#endif
