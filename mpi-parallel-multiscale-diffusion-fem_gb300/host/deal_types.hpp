// deal_types.hpp -- the few deal.II types the reference's local-basis
// interface is written in (Point, Tensor<2,dim>, FullMatrix, Vector, CellId,
// an active-cell handle), restated minimally so the mirror of
// DiffusionProblemBasis compiles without deal.II.  Names and member
// functions follow deal.II's so code written against the reference reads the
// same.
#pragma once

#include <array>
#include <cassert>
#include <stdexcept>
#include <string>
#include <vector>

namespace dealii {

template <int dim>
class Point {
 public:
  Point() { c_.fill(0.0); }
  Point(double x, double y) : Point() { c_[0] = x; c_[1] = y; }
  Point(double x, double y, double z) : Point() { c_[0] = x; c_[1] = y; if (dim > 2) c_[2] = z; }
  double operator()(unsigned int i) const { return c_[i]; }
  double &operator()(unsigned int i) { return c_[i]; }

 private:
  std::array<double, dim> c_;
};

template <int rank, int dim>
class Tensor {
 public:
  Tensor() { clear(); }
  void clear() {
    for (auto &r : v_) r.fill(0.0);
  }
  std::array<double, dim> &operator[](unsigned int i) { return v_[i]; }
  const std::array<double, dim> &operator[](unsigned int i) const { return v_[i]; }

 private:
  std::array<std::array<double, dim>, dim> v_;
};

class FullMatrix {
 public:
  FullMatrix(unsigned int m = 0, unsigned int n = 0) : m_(m), n_(n), v_(size_t(m) * n, 0.0) {}
  double &operator()(unsigned int i, unsigned int j) { return v_[size_t(i) * n_ + j]; }
  double operator()(unsigned int i, unsigned int j) const { return v_[size_t(i) * n_ + j]; }
  unsigned int m() const { return m_; }
  unsigned int n() const { return n_; }
  FullMatrix &operator=(double s) {
    for (auto &x : v_) x = s;
    return *this;
  }

 private:
  unsigned int m_, n_;
  std::vector<double> v_;
};

class Vector {
 public:
  Vector(size_t n = 0) : v_(n, 0.0) {}
  void reinit(size_t n) { v_.assign(n, 0.0); }
  size_t size() const { return v_.size(); }
  double &operator()(size_t i) { return v_[i]; }
  double operator()(size_t i) const { return v_[i]; }
  double *data() { return v_.data(); }
  const double *data() const { return v_.data(); }
  // this = s * this + a * w   (deal.II Vector::sadd)
  void sadd(double s, double a, const Vector &w) {
    for (size_t i = 0; i < v_.size(); ++i) v_[i] = s * v_[i] + a * w.v_[i];
  }

 private:
  std::vector<double> v_;
};

// CellId of a coarse cell (its index in the coarse mesh, written as deal.II
// writes level-0 ids: "<index>_0:").
class CellId {
 public:
  CellId(unsigned int index = 0) : index_(index) {}
  std::string to_string() const { return std::to_string(index_) + "_0:"; }
  bool operator<(const CellId &o) const { return index_ < o.index_; }
  bool operator==(const CellId &o) const { return index_ == o.index_; }
  unsigned int index() const { return index_; }

 private:
  unsigned int index_;
};

using MPI_Comm = int;

// Active coarse cell: vertices in deal.II order (v = vx + 2 vy + 4 vz) and
// its id -- what DiffusionProblemBasis reads from
// Triangulation<dim>::active_cell_iterator.
template <int dim>
class CoarseCell {
 public:
  CoarseCell(unsigned int index, const std::vector<Point<dim>> &vertices)
      : id_(index), v_(vertices) {
    if (v_.size() != (1u << dim)) throw std::invalid_argument("a coarse cell has 2^dim vertices");
  }
  const Point<dim> &vertex(unsigned int i) const { return v_[i]; }
  CellId id() const { return id_; }
  const CoarseCell *operator->() const { return this; }

 private:
  CellId id_;
  std::vector<Point<dim>> v_;
};

template <int dim>
struct GeometryInfo {
  static constexpr unsigned int vertices_per_cell = 1u << dim;
  static constexpr unsigned int faces_per_cell = 2 * dim;
};

}  // namespace dealii
