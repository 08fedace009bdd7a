// msfem_host.cpp -- libmsfem_host.so: the C++ mirror of the reference's
// local-basis and coefficient classes (diffusion_problem_basis.hpp,
// coefficients.hpp) driven by the DiffusionProblemMultiscale replay
// (diffusion_problem_ms.hpp), with a C entry point for tests and callers
// without C++.
#include <cstdio>
#include <cstring>
#include <exception>
#include <memory>
#include <string>

#include "diffusion_problem.hpp"
#include "diffusion_problem_ms.hpp"

namespace {

// A right-hand side without a constant value, f(x) = f0 + x: the batch
// tabulates it at the Gauss points through value_list.
template <int dim>
class LinearRhs : public Coefficients::ScalarFunction<dim> {
 public:
  explicit LinearRhs(double f0) : f0_(f0) {}
  double value(const dealii::Point<dim> &p, unsigned int = 0) const override { return f0_ + p(0); }

 private:
  double f0_;
};

enum { kOptRelativeTol = 1, kOptLinearRhs = 2, kOptOutputBasis = 4 };

// Problem data of every flush: device, precision, coefficient, right-hand
// side and stopping rule.
template <int dim>
void configure(int coef, const double *params, double f_value, int precision, int device, int options) {
  using namespace DiffusionProblem;
  auto &batch = BasisBatch<dim>::get();
  batch.set_device(device);
  batch.set_precision(precision);
  if (options & kOptLinearRhs)
    batch.set_right_hand_side(std::make_shared<LinearRhs<dim>>(f_value));
  else
    batch.set_right_hand_side(f_value);
  batch.set_tolerance(1e-12, 1000, !(options & kOptRelativeTol));
  if (coef == 0) {
    batch.set_coefficient(std::make_shared<Coefficients::MatrixCoeff<dim>>());
  } else if (coef == 1) {
    batch.set_coefficient(std::make_shared<Coefficients::SinSinCoeff<dim>>(params[0], params[1]));
  } else {
    // a coefficient without a device description: tabulated via value_list
    dealii::Tensor<2, dim> A;
    int k = 0;
    for (int i = 0; i < dim; ++i)
      for (int j = i; j < dim; ++j, ++k) A[i][j] = A[j][i] = params[k];
    batch.set_coefficient(std::make_shared<Coefficients::ConstantCoeff<dim>>(A));
  }
}

template <int dim>
int run_ms(int n_refine, int n_refine_local, int coef, const double *params, double f_value, int bc,
           int precision, int device, double *u_out, double *M_out, double *F_out, double *fine_out,
           int write_vtu, int options) {
  using namespace DiffusionProblem;
  configure<dim>(coef, params, f_value, precision, device, options);
  DiffusionProblemMultiscale<dim> ms(n_refine, n_refine_local, bc);
  ms.set_output_flag_first_cell(options & kOptOutputBasis);
  ms.run();
  const auto &u = ms.coarse_solution();
  if (u_out) std::memcpy(u_out, u.data(), sizeof(double) * u.size());
  constexpr unsigned int nv = dealii::GeometryInfo<dim>::vertices_per_cell;
  size_t c = 0;
  for (const auto &cell : ms.cells()) {
    const auto &b = ms.basis_map().at(cell.id());
    const auto &M = b.get_global_element_matrix();
    const auto &F = b.get_global_element_rhs();
    for (unsigned int i = 0; i < nv; ++i) {
      if (M_out)
        for (unsigned int j = 0; j < nv; ++j) M_out[(c * nv + i) * nv + j] = M(i, j);
      if (F_out) F_out[c * nv + i] = F(i);
    }
    if (fine_out) {
      const auto &g = b.global_solution_vector();
      std::memcpy(fine_out + c * b.n_nodes(), g.data(), sizeof(double) * g.size());
    }
    if (write_vtu && c == 0) b.output_global_solution_in_cell();  // into the working directory
    ++c;
  }
  return 0;
}

template <int dim>
int run_fem(int n_refine, int coef, const double *params, double f_value, int bc, int precision, int device,
            double *u_out, int write_vtu, int options) {
  configure<dim>(coef, params, f_value, precision, device, options);
  DiffusionProblem::DiffusionProblem<dim> fem(n_refine, bc);
  fem.run();
  const auto &u = fem.solution();
  if (u_out) std::memcpy(u_out, u.data(), sizeof(double) * u.size());
  if (write_vtu) fem.output_results();  // into the working directory
  return 0;
}

thread_local std::string g_err;

}  // namespace

extern "C" {

// Run the multiscale driver replay on a unit square/cube with 2^n_refine
// coarse cells per direction and 2^n_refine_local fine cells per coarse cell.
//   coef 0: reference MatrixCoeff; 1: SinSin (params amp, eps); 2: constant
//   tensor params (a11,a12,[a13,]a22,...) passed through value_list tabulation.
//   bc 0: reference boundary conditions; 1: homogeneous Dirichlet.
// Outputs (nullable): u [(K+1)^d] coarse solution, M [cells][2^d][2^d],
// F [cells][2^d], fine [cells][(N+1)^d] reconstructed fine solution;
// write_vtu: the first cell's fine solution as VTU in the working directory.
// options: bit 0 = stop at 1e-12 relative instead of the reference's absolute
// 1e-12; bit 1 = f(x) = f_value + x, a right-hand side tabulated through
// value_list; bit 2 = set_output_flag(true) on the first cell (its basis
// functions as VTU in the working directory).
int msfem_host_ms_run(int dim, int n_refine, int n_refine_local, int coef, const double *params,
                      double f_value, int bc, int precision, int device, double *u_out, double *M_out,
                      double *F_out, double *fine_out, int write_vtu, int options) {
  try {
    if (dim == 2)
      return run_ms<2>(n_refine, n_refine_local, coef, params, f_value, bc, precision, device, u_out,
                       M_out, F_out, fine_out, write_vtu, options);
    if (dim == 3)
      return run_ms<3>(n_refine, n_refine_local, coef, params, f_value, bc, precision, device, u_out,
                       M_out, F_out, fine_out, write_vtu, options);
    g_err = "dim must be 2 or 3";
    return -1;
  } catch (const std::exception &e) {
    g_err = e.what();
    return -2;
  }
}

// The standard Q1 FEM on the unit square/cube with 2^n_refine cells per
// direction (DiffusionProblem<dim>::run, diffusion_problem.tpp:336-377): the
// comparator the reference runs beside the MsFEM.  coef, params, f_value, bc,
// precision, device and options as for msfem_host_ms_run; u [(K+1)^d]
// lexicographic nodal solution; write_vtu: solution-std_<d>d_refinements-<n>
// .0000.vtu in the working directory.
int msfem_host_fem_run(int dim, int n_refine, int coef, const double *params, double f_value, int bc,
                       int precision, int device, double *u_out, int write_vtu, int options) {
  try {
    if (dim == 2) return run_fem<2>(n_refine, coef, params, f_value, bc, precision, device, u_out, write_vtu, options);
    if (dim == 3) return run_fem<3>(n_refine, coef, params, f_value, bc, precision, device, u_out, write_vtu, options);
    g_err = "dim must be 2 or 3";
    return -1;
  } catch (const std::exception &e) {
    g_err = e.what();
    return -2;
  }
}

int msfem_host_last_error(char *buf, size_t len) {
  if (!buf || !len) return -1;
  std::snprintf(buf, len, "%s", g_err.c_str());
  return 0;
}

}  // extern "C"
