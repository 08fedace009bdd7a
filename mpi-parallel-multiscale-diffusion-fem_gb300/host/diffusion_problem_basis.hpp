// diffusion_problem_basis.hpp -- host mirror of the reference's
// DiffusionProblem::DiffusionProblemBasis<dim>
// (include/base/diffusion_problem_basis.hpp:68-281), same public API, with
// the computation moved to libmsfem_gpu.so.
//
// The reference's driver calls run() once per owned cell in a serial loop
// (include/base/diffusion_problem_ms.tpp:81-87) and reads the results later
// (:200-201, :322).  So run() only enqueues the cell into a per-rank batch;
// the first getter on any pending object flushes the whole batch in one GPU
// launch and scatters M, F and the basis back into the objects.
#pragma once

#include <cstdio>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "coefficients.hpp"
#include "deal_types.hpp"
#include "msfem_gpu.h"

namespace DiffusionProblem {
using namespace dealii;

template <int dim>
class DiffusionProblemBasis;

// Per-rank batch of pending basis objects (one MPI rank = one GPU).
template <int dim>
class BasisBatch {
 public:
  static BasisBatch &get() {
    static BasisBatch b;
    return b;
  }
  // The handle lives until the process exits (the CUDA context is released
  // then); destroying it from a static destructor could run after the CUDA
  // runtime has shut down.
  void release() {
    if (handle_) msfem_destroy(handle_);
    handle_ = nullptr;
  }
  // Problem data used by every flush (the reference hard-codes MatrixCoeff
  // and RightHandSide inside assemble_system, diffusion_problem_basis.tpp:182-188).
  void set_coefficient(std::shared_ptr<Coefficients::TensorFunction2<dim>> c) { coef_ = std::move(c); }
  // Any Function<dim>: a constant one is passed as f_value, any other is
  // tabulated at the QGauss(2) points through value_list.
  void set_right_hand_side(std::shared_ptr<Coefficients::ScalarFunction<dim>> f) { rhs_ = std::move(f); }
  void set_right_hand_side(double f) { rhs_ = std::make_shared<Coefficients::RightHandSide<dim>>(f); }
  void set_precision(int precision) { precision_ = precision; }
  // absolute = true is the reference's SolverControl(maxit, tol) stop on the
  // l2 norm of the residual; false stops at tol times ||b||.
  void set_tolerance(double tol, int maxit, bool absolute = true) {
    tol_ = tol;
    maxit_ = maxit;
    tol_absolute_ = absolute;
  }
  void set_device(int device) { device_ = device; }
  const msfem_stats &last_stats() const { return stats_; }

  void enqueue(DiffusionProblemBasis<dim> *b) { pending_.push_back(b); }
  void forget(DiffusionProblemBasis<dim> *b) {
    for (auto &p : pending_)
      if (p == b) p = nullptr;
  }
  void flush();

 private:
  BasisBatch()
      : coef_(std::make_shared<Coefficients::MatrixCoeff<dim>>()),
        rhs_(std::make_shared<Coefficients::RightHandSide<dim>>()) {}
  // Gauss points (QGauss(2), x fastest) of every fine cell of a cell with
  // corners cr[2^dim][dim] and N fine cells per direction, for point q.
  static void gauss_points(const double *cr, int N, int q, std::vector<Point<dim>> &pts) {
    constexpr int nv = GeometryInfo<dim>::vertices_per_cell;
    const double g[2] = {0.5 - 0.5 / std::sqrt(3.0), 0.5 + 0.5 / std::sqrt(3.0)};
    const int nfc = dim == 2 ? N * N : N * N * N;
    pts.resize((size_t)nfc);
    for (int fc = 0; fc < nfc; ++fc) {
      const int ci[3] = {fc % N, (fc / N) % N, dim == 3 ? fc / (N * N) : 0};
      double t[3], x[3] = {0, 0, 0};
      for (int a = 0; a < dim; ++a) t[a] = (ci[a] + g[(q >> a) & 1]) / N;
      for (int v = 0; v < nv; ++v) {
        double w = 1.0;
        for (int a = 0; a < dim; ++a) w *= ((v >> a) & 1) ? t[a] : 1.0 - t[a];
        for (int a = 0; a < dim; ++a) x[a] += w * cr[v * dim + a];
      }
      Point<dim> p;
      for (int a = 0; a < dim; ++a) p(a) = x[a];
      pts[fc] = p;
    }
  }
  msfem_handle *handle_ = nullptr;
  std::vector<DiffusionProblemBasis<dim> *> pending_;
  std::shared_ptr<Coefficients::TensorFunction2<dim>> coef_;
  // Coefficients::RightHandSide, f = 2 (right_hand_side.tpp:22)
  std::shared_ptr<Coefficients::ScalarFunction<dim>> rhs_;
  int precision_ = MSFEM_PREC_FP64;
  // SolverControl(1000, 1e-12), diffusion_problem_basis.tpp:297: absolute l2 residual
  double tol_ = 1e-12;
  bool tol_absolute_ = true;
  int maxit_ = 1000;
  int device_ = 0;
  msfem_stats stats_{};
};

template <int dim>
class DiffusionProblemBasis {
 public:
  DiffusionProblemBasis() = delete;

  DiffusionProblemBasis(unsigned int n_refine_local, const CoarseCell<dim> &global_cell,
                        unsigned int local_subdomain, MPI_Comm mpi_communicator)
      : mpi_communicator(mpi_communicator),
        corner_points(GeometryInfo<dim>::vertices_per_cell),
        global_element_matrix(GeometryInfo<dim>::vertices_per_cell, GeometryInfo<dim>::vertices_per_cell),
        global_element_rhs(GeometryInfo<dim>::vertices_per_cell),
        global_weights(GeometryInfo<dim>::vertices_per_cell, 0.0),
        n_refine_local(n_refine_local),
        global_cell_id(global_cell.id()),
        local_subdomain(local_subdomain),
        basis_q1(global_cell) {
    for (unsigned int v = 0; v < GeometryInfo<dim>::vertices_per_cell; ++v)
      corner_points[v] = global_cell.vertex(v);
  }

  DiffusionProblemBasis(const DiffusionProblemBasis &X) = default;

  ~DiffusionProblemBasis() { BasisBatch<dim>::get().forget(this); }

  // diffusion_problem_basis.tpp:438-474
  void run() {
    set_filename_global();
    is_built_global_element_matrix = false;
    BasisBatch<dim>::get().enqueue(this);
  }

  void output_global_solution_in_cell() const {
    if (!is_set_global_weights) throw std::logic_error("Global weights must be set first.");
    write_vtu(filename_global, global_solution);
  }

  const FullMatrix &get_global_element_matrix() const {
    ensure_built();
    return global_element_matrix;
  }

  const Vector &get_global_element_rhs() const {
    ensure_built();
    return global_element_rhs;
  }

  const std::string &get_filename_global() { return filename_global; }

  // diffusion_problem_basis.tpp:352-377: global_solution = sum_i w_i phi_i
  void set_global_weights(const std::vector<double> &weights) {
    ensure_built();
    global_weights = weights;
    global_solution.reinit(n_nodes());
    for (unsigned int i = 0; i < GeometryInfo<dim>::vertices_per_cell; ++i)
      global_solution.sadd(1.0, global_weights[i], solution_vector[i]);
    is_set_global_weights = true;
  }

  void set_output_flag(bool flag) { output_flag = flag; }

  // -- accessors used by the batch (not part of the reference API) --------
  unsigned int n_fine() const { return 1u << n_refine_local; }
  size_t n_nodes() const {
    size_t n = n_fine() + 1, s = 1;
    for (int a = 0; a < dim; ++a) s *= n;
    return s;
  }
  const std::vector<Point<dim>> &corners() const { return corner_points; }
  const Vector &basis(unsigned int i) const { return solution_vector[i]; }
  const Vector &global_solution_vector() const { return global_solution; }

 private:
  friend class BasisBatch<dim>;

  void ensure_built() const {
    if (!is_built_global_element_matrix) BasisBatch<dim>::get().flush();
    if (!is_built_global_element_matrix) throw std::logic_error("run() was not called on this basis object");
  }

  // diffusion_problem_basis.tpp:380-389
  void set_filename_global() {
    char sub[16];
    std::snprintf(sub, sizeof sub, "%05u", local_subdomain);
    filename_global = std::string(dim == 2 ? "solution-ms_fine-2d" : "solution-ms_fine-3d") + "." +
                      sub + ".cell-" + global_cell_id.to_string() + ".vtu";
  }

  // diffusion_problem_basis.tpp:392-418: every basis function of the cell
  // as point data basis_0 .. basis_{2^dim-1} in "2d-basis.<subdomain>.cell-<id>.vtu"
  // ("3d-..." in 3D).  The subdomain field is that of the local serial
  // Triangulation, whose locally_owned_subdomain() is
  // numbers::invalid_subdomain_id (4294967295), as in the reference.
  void output_basis() const {
    std::string name = std::string(dim == 2 ? "2d-" : "3d-") + "basis." + std::to_string(4294967295u) +
                       ".cell-" + global_cell_id.to_string() + ".vtu";
    std::vector<std::pair<std::string, const Vector *>> fields;
    for (unsigned int i = 0; i < GeometryInfo<dim>::vertices_per_cell; ++i)
      fields.emplace_back("basis_" + std::to_string(i), &solution_vector[i]);
    write_vtu(name, fields);
  }

  void write_vtu(const std::string &name, const Vector &field) const { write_vtu(name, {{"solution", &field}}); }

  // Plain VTU of the local fine grid with point fields (replaces DataOut).
  void write_vtu(const std::string &name, const std::vector<std::pair<std::string, const Vector *>> &fields) const {
    const unsigned int N = n_fine(), n = N + 1;
    const size_t nn = n_nodes(), nc = dim == 2 ? size_t(N) * N : size_t(N) * N * N;
    std::ofstream out(name);
    out << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\">\n<UnstructuredGrid>\n";
    out << "<Piece NumberOfPoints=\"" << nn << "\" NumberOfCells=\"" << nc << "\">\n<Points>\n";
    out << "<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
    for (size_t k = 0; k < nn; ++k) {
      double t[3] = {double(k % n) / N, double((k / n) % n) / N, dim == 3 ? double(k / (n * n)) / N : 0.0};
      double x[3] = {0, 0, 0};
      for (unsigned int v = 0; v < GeometryInfo<dim>::vertices_per_cell; ++v) {
        double w = 1.0;
        for (int a = 0; a < dim; ++a) w *= ((v >> a) & 1) ? t[a] : 1.0 - t[a];
        for (int a = 0; a < dim; ++a) x[a] += w * corner_points[v](a);
      }
      out << x[0] << ' ' << x[1] << ' ' << x[2] << '\n';
    }
    out << "</DataArray>\n</Points>\n<Cells>\n<DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n";
    for (size_t c = 0; c < nc; ++c) {
      const size_t cx = c % N, cy = (c / N) % N, cz = dim == 3 ? c / (size_t(N) * N) : 0;
      auto id = [&](size_t i, size_t j, size_t k) { return (k * n + j) * n + i; };
      if (dim == 2)
        out << id(cx, cy, 0) << ' ' << id(cx + 1, cy, 0) << ' ' << id(cx + 1, cy + 1, 0) << ' '
            << id(cx, cy + 1, 0) << '\n';
      else
        out << id(cx, cy, cz) << ' ' << id(cx + 1, cy, cz) << ' ' << id(cx + 1, cy + 1, cz) << ' '
            << id(cx, cy + 1, cz) << ' ' << id(cx, cy, cz + 1) << ' ' << id(cx + 1, cy, cz + 1) << ' '
            << id(cx + 1, cy + 1, cz + 1) << ' ' << id(cx, cy + 1, cz + 1) << '\n';
    }
    out << "</DataArray>\n<DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n";
    const int npc = dim == 2 ? 4 : 8;
    for (size_t c = 0; c < nc; ++c) out << (c + 1) * npc << '\n';
    out << "</DataArray>\n<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n";
    for (size_t c = 0; c < nc; ++c) out << (dim == 2 ? 9 : 12) << '\n';
    out << "</DataArray>\n</Cells>\n<PointData Scalars=\"" << fields[0].first << "\">\n";
    out.precision(17);
    for (const auto &f : fields) {
      out << "<DataArray type=\"Float64\" Name=\"" << f.first << "\" format=\"ascii\">\n";
      for (size_t k = 0; k < nn; ++k) out << (*f.second)(k) << '\n';
      out << "</DataArray>\n";
    }
    out << "</PointData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n";
  }

  MPI_Comm mpi_communicator;
  std::vector<Point<dim>> corner_points;
  std::string filename_global;
  std::vector<Vector> solution_vector;  // basis i at the fine nodes (lexicographic)
  FullMatrix global_element_matrix;
  bool is_built_global_element_matrix = false;
  Vector global_element_rhs;
  std::vector<double> global_weights;
  bool is_set_global_weights = false;
  Vector global_solution;
  unsigned int n_refine_local;
  CellId global_cell_id;
  unsigned int local_subdomain;
  Coefficients::BasisQ1<dim> basis_q1;
  bool output_flag = false;
};

template <int dim>
void BasisBatch<dim>::flush() {
  std::vector<DiffusionProblemBasis<dim> *> cells;
  for (auto *p : pending_)
    if (p) cells.push_back(p);
  pending_.clear();
  if (cells.empty()) return;
  if (!handle_) {
    const int rc = msfem_create(&handle_, device_);
    if (rc != MSFEM_OK) {
      char msg[512];
      msfem_last_error(msg, sizeof msg);
      throw std::runtime_error(std::string("msfem_create: ") + msg);
    }
  }
  constexpr int nv = GeometryInfo<dim>::vertices_per_cell;
  const int n = (int)cells.size();
  std::vector<double> corners((size_t)n * nv * dim);
  std::vector<int32_t> nf(n);
  bool uniform = true;
  for (int c = 0; c < n; ++c) {
    for (int v = 0; v < nv; ++v)
      for (int a = 0; a < dim; ++a) corners[((size_t)c * nv + v) * dim + a] = cells[c]->corners()[v](a);
    nf[c] = (int32_t)cells[c]->n_fine();
    uniform = uniform && nf[c] == nf[0];
  }
  msfem_batch_desc d{};
  d.dim = dim;
  d.n_cells = n;
  d.n_fine = nf[0];
  d.n_fine_per_cell = uniform ? nullptr : nf.data();
  d.precision = precision_;
  d.corners = corners.data();
  d.tol = tol_;
  d.tol_absolute = tol_absolute_ ? 1 : 0;
  d.maxit = maxit_;
  d.memory = MSFEM_MEM_HOST;
  // right-hand side: RightHandSide::value_list at the QGauss(2) points
  // (diffusion_problem_basis.tpp:204-205) unless it is a constant
  std::vector<double> ftab;
  std::vector<int64_t> foff;
  double fconst = 0.0;
  if (rhs_->constant_value(fconst)) {
    d.f_value = fconst;
  } else {
    foff.resize(n);
    std::vector<Point<dim>> pts;
    std::vector<double> vals;
    for (int c = 0; c < n; ++c) {
      const int N = nf[c];
      const int nfc = dim == 2 ? N * N : N * N * N;
      foff[c] = (int64_t)ftab.size();
      ftab.resize(ftab.size() + (size_t)nv * nfc);
      for (int q = 0; q < nv; ++q) {
        gauss_points(corners.data() + (size_t)c * nv * dim, N, q, pts);
        vals.resize(pts.size());
        rhs_->value_list(pts, vals);
        std::copy(vals.begin(), vals.end(), ftab.begin() + foff[c] + (size_t)q * nfc);
      }
    }
    d.f_qp_values = ftab.data();
    d.f_qp_offset = foff.data();
  }
  std::vector<double> tab;
  std::vector<int64_t> qoff;
  if (!coef_->describe(d.coef)) {
    // generic TensorFunction: tabulate at the QGauss(2) points via value_list
    const int ncomp = dim == 2 ? 3 : 6;
    qoff.resize(n);
    for (int c = 0; c < n; ++c) {
      const int N = nf[c];
      const int nfc = dim == 2 ? N * N : N * N * N;
      qoff[c] = (int64_t)tab.size();
      tab.resize(tab.size() + (size_t)ncomp * nv * nfc);
      std::vector<Point<dim>> pts;
      std::vector<Tensor<2, dim>> vals((size_t)nfc);
      for (int q = 0; q < nv; ++q) {
        gauss_points(corners.data() + (size_t)c * nv * dim, N, q, pts);
        coef_->value_list(pts, vals);
        for (int fc = 0; fc < nfc; ++fc) {
          const auto &A = vals[fc];
          double comp[6];
          if (dim == 2) { comp[0] = A[0][0]; comp[1] = A[0][1]; comp[2] = A[1][1]; }
          else { comp[0] = A[0][0]; comp[1] = A[0][1]; comp[2] = A[0][2];
                 comp[3] = A[1][1]; comp[4] = A[1][2]; comp[5] = A[2][2]; }
          for (int k = 0; k < ncomp; ++k) tab[qoff[c] + ((size_t)k * nv + q) * nfc + fc] = comp[k];
        }
      }
    }
    d.coef.kind = MSFEM_COEF_TABULATED;
    d.coef.ncomp = ncomp;
    d.coef.qp_values = tab.data();
    d.coef.qp_offset = qoff.data();
  }
  std::vector<double> M((size_t)n * nv * nv), F((size_t)n * nv);
  size_t basis_total = 0;
  for (auto *c : cells) basis_total += nv * c->n_nodes();
  std::vector<double> basis(basis_total);
  std::vector<int32_t> status(n);
  const int rc = msfem_run_batch(handle_, &d, M.data(), F.data(), basis.data(), status.data(), nullptr, &stats_);
  if (rc != MSFEM_OK) {
    // replaces SolverControl::NoConvergence (diffusion_problem_basis.tpp:297-306)
    char msg[512];
    msfem_last_error(msg, sizeof msg);
    throw std::runtime_error(std::string("msfem_run_batch: ") + msg);
  }
  size_t off = 0;
  for (int c = 0; c < n; ++c) {
    auto *b = cells[c];
    for (int i = 0; i < nv; ++i) {
      for (int j = 0; j < nv; ++j) b->global_element_matrix(i, j) = M[((size_t)c * nv + i) * nv + j];
      b->global_element_rhs(i) = F[(size_t)c * nv + i];
    }
    b->solution_vector.assign(nv, Vector(b->n_nodes()));
    for (int i = 0; i < nv; ++i)
      for (size_t k = 0; k < b->n_nodes(); ++k) b->solution_vector[i](k) = basis[off + i * b->n_nodes() + k];
    off += nv * b->n_nodes();
    b->is_built_global_element_matrix = true;
    // run() writes the basis functions when output_flag is set
    // (diffusion_problem_basis.tpp:468-471)
    if (b->output_flag) b->output_basis();
  }
}

}  // namespace DiffusionProblem
