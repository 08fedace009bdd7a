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
#include <memory>
#include <stdexcept>
#include <vector>

#include "diffusion_problem_basis.hpp"
#include "global_q1.hpp"

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

  // diffusion_problem_ms.tpp:159-255: element matrices and loads from the
  // basis objects (the first getter flushes the GPU batch), Neumann terms,
  // scatter into the global system
  void assemble_system() {
    sys_ = std::make_unique<GlobalQ1System<dim>>(n_cells_per_dir(), bc);
    for (const auto &cell : cells_) {
      const auto &basis = cell_basis_map.at(cell.id());
      sys_->add_cell(cell.id().index(), basis.get_global_element_matrix(), basis.get_global_element_rhs());
    }
  }

  // diffusion_problem_ms.tpp:258-296 (the reference's Trilinos solve): the
  // Dirichlet data and a direct solve
  void solve() { u = sys_->solve(); }

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
  std::unique_ptr<GlobalQ1System<dim>> sys_;
  std::vector<double> u;
};

}  // namespace DiffusionProblem
