// coefficients.hpp -- host-side coefficient classes with the reference's
// interfaces (include/coefficients/*.hpp): value / value_list of a
// TensorFunction<2,dim> or Function<dim>.  Each class can also describe
// itself to the GPU library (msfem_coef_desc); a coefficient that cannot is
// tabulated at the QGauss(2) points through value_list (the generic path).
#pragma once

#include <cmath>
#include <vector>

#include "deal_types.hpp"
#include "msfem_gpu.h"

namespace Coefficients {
using namespace dealii;

// include/coefficients/coefficients.h:21 (the reference's pi constant)
const double PI_D = 3.14592653509793218403;

template <int dim>
class TensorFunction2 {
 public:
  virtual ~TensorFunction2() = default;
  virtual Tensor<2, dim> value(const Point<dim> &p) const = 0;
  virtual void value_list(const std::vector<Point<dim>> &points,
                          std::vector<Tensor<2, dim>> &values) const {
    if (points.size() != values.size()) throw std::invalid_argument("value_list: size mismatch");
    for (size_t i = 0; i < points.size(); ++i) values[i] = value(points[i]);
  }
  // Device description; false = tabulate on the host through value_list.
  virtual bool describe(msfem_coef_desc &d) const {
    (void)d;
    return false;
  }
};

template <int dim>
class ScalarFunction {
 public:
  virtual ~ScalarFunction() = default;
  virtual double value(const Point<dim> &p, unsigned int component = 0) const = 0;
  virtual void value_list(const std::vector<Point<dim>> &points, std::vector<double> &values,
                          unsigned int component = 0) const {
    if (points.size() != values.size()) throw std::invalid_argument("value_list: size mismatch");
    for (size_t i = 0; i < points.size(); ++i) values[i] = value(points[i], component);
  }
  // A constant function reports its value (no tabulation needed).
  virtual bool constant_value(double &v) const {
    (void)v;
    return false;
  }
};

// MatrixCoeff<dim>, include/coefficients/matrix_coeff.tpp:17-91:
// c(x) = 1 - 0.9999 (0.5 sin(2 PI_D 57 x) + 0.5 sin(2 PI_D 57 y)), A = R diag(c) R^T.
template <int dim>
class MatrixCoeff : public TensorFunction2<dim> {
 public:
  MatrixCoeff() {
    const double al = PI_D / 3, be = PI_D / 6, ga = PI_D / 4;
    if (dim == 2) {
      rot_[0][0] = std::cos(al); rot_[0][1] = std::sin(al);
      rot_[1][0] = -std::sin(al); rot_[1][1] = std::cos(al);
    } else {
      rot_[0][0] = std::cos(al) * std::cos(ga) - std::sin(al) * std::cos(be) * std::sin(ga);
      rot_[0][1] = -std::cos(al) * std::sin(ga) - std::sin(al) * std::cos(be) * std::cos(ga);
      rot_[0][2] = std::sin(al) * std::sin(be);
      rot_[1][0] = std::sin(al) * std::cos(ga) + std::cos(al) * std::cos(be) * std::sin(ga);
      rot_[1][1] = -std::sin(al) * std::sin(ga) + std::cos(al) * std::cos(be) * std::cos(ga);
      rot_[1][2] = -std::cos(al) * std::sin(be);
      rot_[2][0] = std::sin(be) * std::sin(ga);
      rot_[2][1] = std::sin(be) * std::cos(ga);
      rot_[2][2] = std::cos(be);
    }
  }
  Tensor<2, dim> value(const Point<dim> &p) const override {
    const double c = 1.0 * (1.0 - 0.9999 * (0.5 * std::sin(2 * PI_D * 57 * p(0)) +
                                            0.5 * std::sin(2 * PI_D * 57 * p(1))));
    Tensor<2, dim> out;
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) {
        double s = 0.0;
        for (int k = 0; k < dim; ++k) s += rot_[i][k] * c * rot_[j][k];
        out[i][j] = s;
      }
    return out;
  }
  bool describe(msfem_coef_desc &d) const override {
    d.kind = MSFEM_COEF_REFERENCE;
    return true;
  }

 private:
  Tensor<2, dim> rot_;
};

// Scalar oscillating coefficient a = 1 + amp sin(2 pi x/eps) sin(2 pi y/eps) [sin z].
template <int dim>
class SinSinCoeff : public TensorFunction2<dim> {
 public:
  SinSinCoeff(double amp, double eps) : amp_(amp), eps_(eps) {}
  Tensor<2, dim> value(const Point<dim> &p) const override {
    const double pi = 3.14159265358979323846;
    double s = std::sin(2 * pi * p(0) / eps_) * std::sin(2 * pi * p(1) / eps_);
    if (dim == 3) s *= std::sin(2 * pi * p(2) / eps_);
    Tensor<2, dim> out;
    for (int i = 0; i < dim; ++i) out[i][i] = 1.0 + amp_ * s;
    return out;
  }
  bool describe(msfem_coef_desc &d) const override {
    d.kind = MSFEM_COEF_SINSIN;
    d.params[0] = amp_;
    d.params[1] = eps_;
    return true;
  }

 private:
  double amp_, eps_;
};

// Any user coefficient (no device description): tabulated through value_list.
template <int dim>
class ConstantCoeff : public TensorFunction2<dim> {
 public:
  explicit ConstantCoeff(const Tensor<2, dim> &a) : a_(a) {}
  Tensor<2, dim> value(const Point<dim> &) const override { return a_; }

 private:
  Tensor<2, dim> a_;
};

// RightHandSide<dim>, right_hand_side.tpp:17-40: f = 2 (value configurable).
template <int dim>
class RightHandSide : public ScalarFunction<dim> {
 public:
  explicit RightHandSide(double f = 2.0) : f_(f) {}
  double value(const Point<dim> &, unsigned int = 0) const override { return f_; }
  double constant() const { return f_; }
  bool constant_value(double &v) const override {
    v = f_;
    return true;
  }

 private:
  double f_;
};

// DirichletBC<dim>, dirichlet_bc.tpp:17-43: (x-1/2)^2 + (y-1/2)^2.
template <int dim>
class DirichletBC : public ScalarFunction<dim> {
 public:
  double value(const Point<dim> &p, unsigned int = 0) const override {
    return (p(0) - 0.5) * (p(0) - 0.5) + (p(1) - 0.5) * (p(1) - 0.5);
  }
};

// NeumannBC<dim>, neumann_bc.tpp:17-41: cos(2 PI_D x) cos(2 PI_D y).
template <int dim>
class NeumannBC : public ScalarFunction<dim> {
 public:
  double value(const Point<dim> &p, unsigned int = 0) const override {
    return std::cos(2 * PI_D * p(0)) * std::cos(2 * PI_D * p(1));
  }
};

// BasisQ1<dim>, basis_q1.tpp:26-158: the 2^dim coarse Q1 nodal functions of
// a cell, set_index selects one.  Built in translated, scaled monomials
// (same polynomial space, well-conditioned Vandermonde matrix).
template <int dim>
class BasisQ1 : public ScalarFunction<dim> {
 public:
  static constexpr int nv = 1 << dim;
  explicit BasisQ1(const CoarseCell<dim> &cell) : index_basis_(0) {
    double H = 0.0;
    for (int a = 0; a < dim; ++a) shift_[a] = cell.vertex(0)(a);
    for (int v = 1; v < nv; ++v)
      for (int a = 0; a < dim; ++a) H = std::max(H, std::fabs(cell.vertex(v)(a) - shift_[a]));
    scale_ = H > 0 ? H : 1.0;
    double w[nv][2 * nv];
    for (int v = 0; v < nv; ++v) {
      double m[nv];
      monomials(cell.vertex(v), m);
      for (int j = 0; j < nv; ++j) {
        w[v][j] = m[j];
        w[v][nv + j] = j == v ? 1.0 : 0.0;
      }
    }
    for (int col = 0; col < nv; ++col) {
      int piv = col;
      for (int r = col + 1; r < nv; ++r)
        if (std::fabs(w[r][col]) > std::fabs(w[piv][col])) piv = r;
      if (w[piv][col] == 0.0) throw std::runtime_error("BasisQ1: degenerate cell");
      for (int j = 0; j < 2 * nv; ++j) std::swap(w[col][j], w[piv][j]);
      const double d = w[col][col];
      for (int j = 0; j < 2 * nv; ++j) w[col][j] /= d;
      for (int r = 0; r < nv; ++r)
        if (r != col) {
          const double f = w[r][col];
          for (int j = 0; j < 2 * nv; ++j) w[r][j] -= f * w[col][j];
        }
    }
    for (int m = 0; m < nv; ++m)
      for (int i = 0; i < nv; ++i) coef_[m][i] = w[m][nv + i];
  }
  void set_index(unsigned int index) { index_basis_ = index; }
  double value(const Point<dim> &p, unsigned int = 0) const override {
    double m[nv];
    monomials(p, m);
    double s = 0.0;
    for (int k = 0; k < nv; ++k) s += coef_[k][index_basis_] * m[k];
    return s;
  }

 private:
  void monomials(const Point<dim> &p, double *m) const {
    double x[3] = {0, 0, 0};
    for (int a = 0; a < dim; ++a) x[a] = (p(a) - shift_[a]) / scale_;
    if (dim == 2) {
      m[0] = 1; m[1] = x[0]; m[2] = x[1]; m[3] = x[0] * x[1];
    } else {
      m[0] = 1; m[1] = x[0]; m[2] = x[1]; m[3] = x[2];
      m[4] = x[0] * x[1]; m[5] = x[1] * x[2]; m[6] = x[0] * x[2]; m[7] = x[0] * x[1] * x[2];
    }
  }
  unsigned int index_basis_;
  double shift_[3] = {0, 0, 0};
  double scale_ = 1.0;
  double coef_[nv][nv];
};

}  // namespace Coefficients
