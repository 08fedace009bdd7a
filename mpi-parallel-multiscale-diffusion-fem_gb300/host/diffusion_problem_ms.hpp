// diffusion_problem_ms.hpp -- a deal.II-free driver that replays the call
// sequence of the reference's DiffusionProblemMultiscale<dim>
// (include/base/diffusion_problem_ms.tpp) on one rank:
//   make_grid (:91-103)                unit cube, n_refine uniform refinements
//   initialize_and_compute_basis (:40-88)  one DiffusionProblemBasis per cell,
//                                      copied into a std::map, run() in a loop
//   assemble_system (:159-255)         M, F per cell + Neumann faces (odd ids)
//   solve (:258-296)                   Dirichlet data on the even ids; the
//                                      reference uses Trilinos CG+AMG, this
//                                      driver a direct Cholesky solve
//   send_global_weights_to_cell (:299-325)
// It is the integration harness of the GPU basis layer; the global solver of
// the real code stays the reference's own.
#pragma once

#include <cmath>
#include <map>
#include <stdexcept>
#include <vector>

#include "diffusion_problem_basis.hpp"

namespace DiffusionProblem {

template <int dim>
class DiffusionProblemMultiscale {
 public:
  // bc = 0: the reference's boundary conditions (DirichletBC on ids 0/2/4,
  // NeumannBC on ids 1/3/5); bc = 1: homogeneous Dirichlet everywhere.
  DiffusionProblemMultiscale(unsigned int n_refine, unsigned int n_refine_local, int bc = 0)
      : n_refine(n_refine), n_refine_local(n_refine_local), bc(bc) {}

  void run() {
    make_grid();
    initialize_and_compute_basis();
    assemble_system();
    solve();
    send_global_weights_to_cell();
  }

  // The reference has no such switch (its driver never calls
  // set_output_flag); the mock driver uses it to exercise output_basis.
  void set_output_flag_first_cell(bool flag) { output_first_ = flag; }

  unsigned int n_cells_per_dir() const { return 1u << n_refine; }
  const std::vector<double> &coarse_solution() const { return u; }
  const std::map<CellId, DiffusionProblemBasis<dim>> &basis_map() const { return cell_basis_map; }
  const std::vector<CoarseCell<dim>> &cells() const { return cells_; }

 private:
  void make_grid() {
    const unsigned int K = n_cells_per_dir();
    size_t nc = 1;
    for (int a = 0; a < dim; ++a) nc *= K;
    cells_.clear();
    for (size_t c = 0; c < nc; ++c) {
      const unsigned int ci[3] = {unsigned(c % K), unsigned((c / K) % K), dim == 3 ? unsigned(c / (K * K)) : 0u};
      std::vector<Point<dim>> v(GeometryInfo<dim>::vertices_per_cell);
      for (unsigned int k = 0; k < GeometryInfo<dim>::vertices_per_cell; ++k)
        for (int a = 0; a < dim; ++a) v[k](a) = double(ci[a] + ((k >> a) & 1)) / K;
      cells_.emplace_back(unsigned(c), v);
    }
  }

  void initialize_and_compute_basis() {
    cell_basis_map.clear();
    for (const auto &cell : cells_) {
      DiffusionProblemBasis<dim> current_cell_problem(n_refine_local, cell, 0, 0);
      if (output_first_ && cell.id() == cells_.front().id()) current_cell_problem.set_output_flag(true);
      auto result = cell_basis_map.insert(std::make_pair(cell.id(), current_cell_problem));
      if (!result.second) throw std::logic_error("Insertion of local basis problem into std::map failed.");
    }
    for (auto &kv : cell_basis_map) kv.second.run();
  }

  size_t node_index(const unsigned int *ijk) const {
    const size_t n = n_cells_per_dir() + 1;
    return ijk[0] + n * (ijk[1] + (dim == 3 ? n * ijk[2] : 0));
  }

  void assemble_system() {
    const unsigned int K = n_cells_per_dir();
    size_t nn = 1;
    for (int a = 0; a < dim; ++a) nn *= (K + 1);
    A.assign(nn * nn, 0.0);
    rhs.assign(nn, 0.0);
    const double g[2] = {0.5 - 0.5 / std::sqrt(3.0), 0.5 + 0.5 / std::sqrt(3.0)};
    Coefficients::NeumannBC<dim> neumann;
    constexpr unsigned int nv = GeometryInfo<dim>::vertices_per_cell;
    for (const auto &cell : cells_) {
      const auto &basis = cell_basis_map.at(cell.id());
      const FullMatrix &M = basis.get_global_element_matrix();  // flushes the GPU batch
      Vector F = basis.get_global_element_rhs();
      const unsigned int c = cell.id().index();
      const unsigned int ci[3] = {c % K, (c / K) % K, dim == 3 ? c / (K * K) : 0u};
      if (bc == 0) {
        // Neumann faces with odd boundary id, QGauss<dim-1>(2) (diffusion_problem_ms.tpp:206-235)
        for (int a = 0; a < dim; ++a) {
          if (ci[a] != K - 1) continue;
          const int nfq = 1 << (dim - 1);
          for (int fq = 0; fq < nfq; ++fq) {
            double xi[3];
            int bt = 0;
            for (int e = 0; e < dim; ++e) {
              if (e == a) { xi[e] = 1.0; continue; }
              xi[e] = g[(fq >> bt) & 1];
              ++bt;
            }
            Point<dim> x;
            for (int e = 0; e < dim; ++e) x(e) = (ci[e] + xi[e]) / K;
            const double gv = neumann.value(x);
            const double JxW = std::pow(1.0 / K, dim - 1) / nfq;
            for (unsigned int i = 0; i < nv; ++i) {
              double psi = 1.0;
              for (int e = 0; e < dim; ++e) psi *= ((i >> e) & 1) ? xi[e] : 1.0 - xi[e];
              F(i) += gv * psi * JxW;
            }
          }
        }
      }
      for (unsigned int i = 0; i < nv; ++i) {
        unsigned int ni[3] = {0, 0, 0};
        for (int a = 0; a < dim; ++a) ni[a] = ci[a] + ((i >> a) & 1);
        const size_t gi = node_index(ni);
        for (unsigned int j = 0; j < nv; ++j) {
          unsigned int nj[3] = {0, 0, 0};
          for (int a = 0; a < dim; ++a) nj[a] = ci[a] + ((j >> a) & 1);
          A[gi * nn + node_index(nj)] += M(i, j);
        }
        rhs[gi] += F(i);
      }
    }
  }

  void solve() {
    const unsigned int K = n_cells_per_dir();
    const size_t nn = rhs.size(), n = K + 1;
    Coefficients::DirichletBC<dim> dirichlet;
    std::vector<double> ud(nn, 0.0);
    std::vector<char> fixed(nn, 0);
    for (size_t g = 0; g < nn; ++g) {
      const unsigned int ijk[3] = {unsigned(g % n), unsigned((g / n) % n), dim == 3 ? unsigned(g / (n * n)) : 0u};
      bool lower = false, any = false;
      Point<dim> x;
      for (int a = 0; a < dim; ++a) {
        x(a) = double(ijk[a]) / K;
        if (ijk[a] == 0) lower = any = true;
        if (ijk[a] == K) any = true;
      }
      if (bc == 0 && lower) { fixed[g] = 1; ud[g] = dirichlet.value(x); }
      if (bc == 1 && any) { fixed[g] = 1; ud[g] = 0.0; }
    }
    std::vector<size_t> freeidx;
    for (size_t g = 0; g < nn; ++g)
      if (!fixed[g]) freeidx.push_back(g);
    const size_t nf = freeidx.size();
    std::vector<double> L(nf * nf), b(nf);
    for (size_t r = 0; r < nf; ++r) {
      double s = rhs[freeidx[r]];
      for (size_t g = 0; g < nn; ++g)
        if (fixed[g]) s -= A[freeidx[r] * nn + g] * ud[g];
      b[r] = s;
      for (size_t c = 0; c < nf; ++c) L[r * nf + c] = A[freeidx[r] * nn + freeidx[c]];
    }
    // dense Cholesky (coarse systems here are small)
    for (size_t j = 0; j < nf; ++j) {
      double s = L[j * nf + j];
      for (size_t k = 0; k < j; ++k) s -= L[j * nf + k] * L[j * nf + k];
      if (!(s > 0)) throw std::runtime_error("coarse matrix not positive definite");
      const double d = std::sqrt(s);
      L[j * nf + j] = d;
      for (size_t i = j + 1; i < nf; ++i) {
        double t = L[i * nf + j];
        for (size_t k = 0; k < j; ++k) t -= L[i * nf + k] * L[j * nf + k];
        L[i * nf + j] = t / d;
      }
    }
    for (size_t i = 0; i < nf; ++i) {
      double s = b[i];
      for (size_t k = 0; k < i; ++k) s -= L[i * nf + k] * b[k];
      b[i] = s / L[i * nf + i];
    }
    for (size_t i = nf; i-- > 0;) {
      double s = b[i];
      for (size_t k = i + 1; k < nf; ++k) s -= L[k * nf + i] * b[k];
      b[i] = s / L[i * nf + i];
    }
    u = ud;
    for (size_t r = 0; r < nf; ++r) u[freeidx[r]] = b[r];
  }

  void send_global_weights_to_cell() {
    const unsigned int K = n_cells_per_dir();
    constexpr unsigned int nv = GeometryInfo<dim>::vertices_per_cell;
    for (const auto &cell : cells_) {
      const unsigned int c = cell.id().index();
      const unsigned int ci[3] = {c % K, (c / K) % K, dim == 3 ? c / (K * K) : 0u};
      std::vector<double> w(nv);
      for (unsigned int i = 0; i < nv; ++i) {
        unsigned int ni[3] = {0, 0, 0};
        for (int a = 0; a < dim; ++a) ni[a] = ci[a] + ((i >> a) & 1);
        w[i] = u[node_index(ni)];
      }
      cell_basis_map.at(cell.id()).set_global_weights(w);
    }
  }

  unsigned int n_refine, n_refine_local;
  int bc;
  std::vector<CoarseCell<dim>> cells_;
  std::map<CellId, DiffusionProblemBasis<dim>> cell_basis_map;
  bool output_first_ = false;
  std::vector<double> A, rhs, u;
};

}  // namespace DiffusionProblem
