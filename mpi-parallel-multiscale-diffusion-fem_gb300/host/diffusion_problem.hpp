// diffusion_problem.hpp -- host mirror of the reference's standard FEM,
// DiffusionProblem::DiffusionProblem<dim> (include/base/diffusion_problem.hpp:
// 86-169, include/base/diffusion_problem.tpp:102-377): Q1 FEM for
// -div(A grad u) = f on the unit square / cube refined n_refine times, with
// the same coefficient, right-hand side and boundary data as the MsFEM.  The
// reference runs it beside the MsFEM to measure the multiscale method's
// error (source/main.cxx:33-35).
//
// No separate assembler: a coarse cell with one fine cell per direction
// (N = 1) has no interior nodes, so its multiscale basis is the Q1 basis and
// the GPU batch call returns exactly the standard QGauss(2) element matrices
// and loads (diffusion_problem.tpp:159-236).  The global assembly, the
// Neumann faces, the Dirichlet data and the direct solve are those of the
// MsFEM replay (GlobalQ1System); the reference solves with Trilinos CG + AMG.
#pragma once

#include <fstream>
#include <string>
#include <vector>

#include "diffusion_problem_ms.hpp"

namespace DiffusionProblem {

template <int dim>
class DiffusionProblem {
 public:
  // bc = 0: the reference's boundary data; 1: homogeneous Dirichlet.
  explicit DiffusionProblem(unsigned int n_refine, int bc = 0) : n_refine(n_refine), fine_(n_refine, 0, bc) {}

  // diffusion_problem.tpp:336-377: grid, element matrices on the GPU,
  // assembly, solve
  void run() { fine_.run(); }

  // Nodal solution on the (2^n_refine + 1)^dim grid, lexicographic.
  const std::vector<double> &solution() const { return fine_.coarse_solution(); }

  // diffusion_problem.tpp:283-333: "solution-std_<dim>d_refinements-<n>.0000.vtu"
  // with the point field "u" (one rank: subdomain 0).
  void output_results() const {
    const unsigned int K = 1u << n_refine, n = K + 1;
    const size_t nn = dim == 2 ? size_t(n) * n : size_t(n) * n * n;
    const size_t nc = dim == 2 ? size_t(K) * K : size_t(K) * K * K;
    const std::string name = std::string(dim == 2 ? "solution-std_2d" : "solution-std_3d") + "_refinements-" +
                             std::to_string(n_refine) + ".0000.vtu";
    std::ofstream out(name);
    out.precision(17);
    out << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\">\n<UnstructuredGrid>\n";
    out << "<Piece NumberOfPoints=\"" << nn << "\" NumberOfCells=\"" << nc << "\">\n<Points>\n";
    out << "<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
    for (size_t k = 0; k < nn; ++k)
      out << double(k % n) / K << ' ' << double((k / n) % n) / K << ' '
          << (dim == 3 ? double(k / (size_t(n) * n)) / K : 0.0) << '\n';
    out << "</DataArray>\n</Points>\n<Cells>\n<DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n";
    for (size_t c = 0; c < nc; ++c) {
      const size_t cx = c % K, cy = (c / K) % K, cz = dim == 3 ? c / (size_t(K) * K) : 0;
      auto id = [&](size_t i, size_t j, size_t k) { return (k * n + j) * n + i; };
      if (dim == 2)
        out << id(cx, cy, 0) << ' ' << id(cx + 1, cy, 0) << ' ' << id(cx + 1, cy + 1, 0) << ' ' << id(cx, cy + 1, 0)
            << '\n';
      else
        out << id(cx, cy, cz) << ' ' << id(cx + 1, cy, cz) << ' ' << id(cx + 1, cy + 1, cz) << ' '
            << id(cx, cy + 1, cz) << ' ' << id(cx, cy, cz + 1) << ' ' << id(cx + 1, cy, cz + 1) << ' '
            << id(cx + 1, cy + 1, cz + 1) << ' ' << id(cx, cy + 1, cz + 1) << '\n';
    }
    out << "</DataArray>\n<DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n";
    for (size_t c = 0; c < nc; ++c) out << (c + 1) * (dim == 2 ? 4 : 8) << '\n';
    out << "</DataArray>\n<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n";
    for (size_t c = 0; c < nc; ++c) out << (dim == 2 ? 9 : 12) << '\n';
    out << "</DataArray>\n</Cells>\n<PointData Scalars=\"u\">\n<DataArray type=\"Float64\" Name=\"u\" format=\"ascii\">\n";
    for (double v : solution()) out << v << '\n';
    out << "</DataArray>\n</PointData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n";
  }

 private:
  unsigned int n_refine;
  DiffusionProblemMultiscale<dim> fine_;
};

}  // namespace DiffusionProblem
