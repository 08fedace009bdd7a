// global_q1.hpp -- the global Q1 system on the unit square / cube shared by
// the MsFEM driver replay (diffusion_problem_ms.hpp) and the standard FEM
// (diffusion_problem.hpp): scatter of element matrices and loads, the
// reference's boundary data, and a direct solve.
//
// Coarse mesh: GridGenerator::hyper_cube(0, 1, colorize) refined n_refine
// times, K = 2^n_refine cells per direction, nodes lexicographic (x fastest).
// bc = 0 is the reference's problem: DirichletBC on the faces with even
// boundary id (x = 0, y = 0[, z = 0]) and NeumannBC on the odd ones, integrated
// with QGauss<dim-1>(2) (include/base/diffusion_problem_ms.tpp:129-137,
// :206-235; include/base/diffusion_problem.tpp, same classes); bc = 1 is
// homogeneous Dirichlet on the whole boundary.  The reference solves with
// Trilinos CG + AMG; here the system is stored as a symmetric band (the
// lexicographic numbering gives bandwidth (K+1)^(dim-1) + ... + 1) and solved
// by banded Cholesky, exact to rounding.
#pragma once

#include <cmath>
#include <stdexcept>
#include <vector>

#include "coefficients.hpp"
#include "deal_types.hpp"

namespace DiffusionProblem {
using namespace dealii;

template <int dim>
class GlobalQ1System {
 public:
  GlobalQ1System(unsigned int K, int bc) : K_(K), bc_(bc) {
    const size_t n = K + 1;
    nn_ = dim == 2 ? n * n : n * n * n;
    bw_ = dim == 2 ? n + 1 : n * n + n + 1;
    band_.assign(nn_ * (bw_ + 1), 0.0);
    rhs_.assign(nn_, 0.0);
  }

  size_t n_nodes() const { return nn_; }

  // Node index of vertex i of cell c (c = cx + K (cy + K cz)).
  size_t cell_node(unsigned int c, unsigned int i) const {
    const unsigned int ci[3] = {c % K_, (c / K_) % K_, dim == 3 ? c / (K_ * K_) : 0u};
    const size_t n = K_ + 1;
    size_t g = 0, stride = 1;
    for (int a = 0; a < dim; ++a) {
      g += (ci[a] + ((i >> a) & 1)) * stride;
      stride *= n;
    }
    return g;
  }

  // Adds cell c's element matrix and load (plus its Neumann face terms for
  // bc = 0).
  void add_cell(unsigned int c, const FullMatrix &M, const Vector &F_in) {
    constexpr unsigned int nv = GeometryInfo<dim>::vertices_per_cell;
    Vector F = F_in;
    const unsigned int ci[3] = {c % K_, (c / K_) % K_, dim == 3 ? c / (K_ * K_) : 0u};
    if (bc_ == 0) {
      const double g[2] = {0.5 - 0.5 / std::sqrt(3.0), 0.5 + 0.5 / std::sqrt(3.0)};
      Coefficients::NeumannBC<dim> neumann;
      for (int a = 0; a < dim; ++a) {
        if (ci[a] != K_ - 1) continue;  // only faces on x_a = 1 (odd boundary id)
        const int nfq = 1 << (dim - 1);
        for (int fq = 0; fq < nfq; ++fq) {
          double xi[3];
          int bt = 0;
          for (int e = 0; e < dim; ++e) {
            if (e == a) {
              xi[e] = 1.0;
              continue;
            }
            xi[e] = g[(fq >> bt) & 1];
            ++bt;
          }
          Point<dim> x;
          for (int e = 0; e < dim; ++e) x(e) = (ci[e] + xi[e]) / K_;
          const double gv = neumann.value(x);
          const double JxW = std::pow(1.0 / K_, dim - 1) / nfq;
          for (unsigned int i = 0; i < nv; ++i) {
            double psi = 1.0;
            for (int e = 0; e < dim; ++e) psi *= ((i >> e) & 1) ? xi[e] : 1.0 - xi[e];
            F(i) += gv * psi * JxW;
          }
        }
      }
    }
    for (unsigned int i = 0; i < nv; ++i) {
      const size_t gi = cell_node(c, i);
      for (unsigned int j = 0; j < nv; ++j) {
        const size_t gj = cell_node(c, j);
        if (gj <= gi) band_[gi * (bw_ + 1) + (gi - gj)] += M(i, j);  // lower triangle
      }
      rhs_[gi] += F(i);
    }
  }

  // Dirichlet data by symmetric elimination, then banded Cholesky.
  std::vector<double> solve() const {
    const size_t n = K_ + 1, W = bw_ + 1;
    std::vector<double> L = band_, b = rhs_, ud(nn_, 0.0);
    std::vector<char> fixed(nn_, 0);
    Coefficients::DirichletBC<dim> dirichlet;
    for (size_t g = 0; g < nn_; ++g) {
      const unsigned int ijk[3] = {unsigned(g % n), unsigned((g / n) % n), dim == 3 ? unsigned(g / (n * n)) : 0u};
      bool lower = false, any = false;
      Point<dim> x;
      for (int a = 0; a < dim; ++a) {
        x(a) = double(ijk[a]) / K_;
        if (ijk[a] == 0) lower = any = true;
        if (ijk[a] == K_) any = true;
      }
      if (bc_ == 0 && lower) { fixed[g] = 1; ud[g] = dirichlet.value(x); }
      if (bc_ == 1 && any) { fixed[g] = 1; ud[g] = 0.0; }
    }
    auto at = [&](size_t i, size_t j) -> double & { return L[i * W + (i - j)]; };  // i >= j, i - j <= bw
    // move the fixed columns to the right-hand side, then make fixed rows identity
    for (size_t i = 0; i < nn_; ++i) {
      if (fixed[i]) continue;
      const size_t j0 = i > bw_ ? i - bw_ : 0;
      for (size_t j = j0; j < i; ++j)
        if (fixed[j]) b[i] -= at(i, j) * ud[j];
      for (size_t j = i + 1; j < std::min(nn_, i + bw_ + 1); ++j)
        if (fixed[j]) b[i] -= at(j, i) * ud[j];
    }
    for (size_t i = 0; i < nn_; ++i) {
      const size_t j0 = i > bw_ ? i - bw_ : 0;
      for (size_t j = j0; j < i; ++j)
        if (fixed[i] || fixed[j]) at(i, j) = 0.0;
      if (fixed[i]) {
        at(i, i) = 1.0;
        b[i] = ud[i];
      }
    }
    // banded Cholesky L L^T in place
    for (size_t j = 0; j < nn_; ++j) {
      const size_t k0 = j > bw_ ? j - bw_ : 0;
      double s = at(j, j);
      for (size_t k = k0; k < j; ++k) s -= at(j, k) * at(j, k);
      if (!(s > 0)) throw std::runtime_error("global matrix not positive definite");
      const double d = std::sqrt(s);
      at(j, j) = d;
      for (size_t i = j + 1; i < std::min(nn_, j + bw_ + 1); ++i) {
        const size_t kk = i > bw_ ? i - bw_ : 0;
        double t = at(i, j);
        for (size_t k = std::max(k0, kk); k < j; ++k) t -= at(i, k) * at(j, k);
        at(i, j) = t / d;
      }
    }
    for (size_t i = 0; i < nn_; ++i) {
      const size_t k0 = i > bw_ ? i - bw_ : 0;
      double s = b[i];
      for (size_t k = k0; k < i; ++k) s -= at(i, k) * b[k];
      b[i] = s / at(i, i);
    }
    for (size_t i = nn_; i-- > 0;) {
      double s = b[i];
      for (size_t k = i + 1; k < std::min(nn_, i + bw_ + 1); ++k) s -= at(k, i) * b[k];
      b[i] = s / at(i, i);
    }
    return b;
  }

 private:
  unsigned int K_;
  int bc_;
  size_t nn_ = 0, bw_ = 0;
  std::vector<double> band_, rhs_;
};

}  // namespace DiffusionProblem
