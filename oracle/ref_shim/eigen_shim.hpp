// eigen_shim.hpp - a small stand-in for the part of the Eigen 3.4 dense API that the reference's
// NNP path uses, so that the reference's own sources compile here without Eigen.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref).  Eigen 3.4-rc1 is a header-only dependency that the
// reference does not vendor (src/Makefile:4) and that this image lacks.  This header restates
// the published semantics of the calls the path makes - column-major dense matrices and vectors
// of fixed or dynamic size, coefficient-wise arithmetic, matrix products, diagonal wrappers,
// norms, dot and cross products, row/column blocks - with eager evaluation and sums in index
// order (a(i,0) b(0,j) + a(i,1) b(1,j) + ...).  Eigen's own kernels may sum dynamic-size
// products in another order (packets, blocking), so results agree with a real Eigen build to
// rounding, not bit for bit; nothing of Eigen's source is used.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <ostream>
#include <stdexcept>
#include <type_traits>
#include <vector>

namespace Eigen {

typedef std::ptrdiff_t Index;
const int Dynamic = -1;
const int Infinity = -1;

template <typename S, int R, int C>
class Matrix;
template <typename M, bool IsRow>
class Block;
template <typename S>
class DiagonalWrapper;

template <typename T>
struct traits;
template <typename S, int R, int C>
struct traits<Matrix<S, R, C>> {
  typedef S Scalar;
  enum { Rows = R, Cols = C };
};
template <typename M, bool IsRow>
struct traits<Block<M, IsRow>> {
  typedef typename std::remove_const<M>::type Base;
  typedef typename traits<Base>::Scalar Scalar;
  enum { Rows = IsRow ? 1 : (int)traits<Base>::Rows, Cols = IsRow ? (int)traits<Base>::Cols : 1 };
};

// Fixed or dynamic dimension of a result: the first fixed one of the operands.
constexpr int pick_dim(int a, int b) { return a != Dynamic ? a : b; }

template <typename Derived>
class DenseBase {
 public:
  typedef typename traits<Derived>::Scalar Scalar;
  enum { RowsAtCompileTime = traits<Derived>::Rows, ColsAtCompileTime = traits<Derived>::Cols };
  typedef Matrix<Scalar, RowsAtCompileTime, ColsAtCompileTime> PlainObject;

  const Derived& derived() const { return static_cast<const Derived&>(*this); }
  Derived& derived() { return static_cast<Derived&>(*this); }
  Index rows() const { return derived().rows(); }
  Index cols() const { return derived().cols(); }
  Index size() const { return rows() * cols(); }
  // linear coefficient of a vector (or column-major position of a matrix)
  Scalar lin(Index k) const {
    const Index r = rows();
    return derived().coeff(k % r, k / r);
  }

  Scalar sum() const {
    Scalar s = 0;
    for (Index k = 0; k < size(); ++k) s += lin(k);
    return s;
  }
  Scalar prod() const {
    Scalar s = 1;
    for (Index k = 0; k < size(); ++k) s *= lin(k);
    return s;
  }
  Scalar squaredNorm() const {
    Scalar s = 0;
    for (Index k = 0; k < size(); ++k) s += lin(k) * lin(k);
    return s;
  }
  Scalar norm() const { return std::sqrt(squaredNorm()); }
  template <int P>
  Scalar lpNorm() const {
    Scalar s = 0;
    if (P == Infinity) {
      for (Index k = 0; k < size(); ++k) s = std::max<Scalar>(s, std::abs(lin(k)));
      return s;
    }
    if (P == 1) {
      for (Index k = 0; k < size(); ++k) s += std::abs(lin(k));
      return s;
    }
    for (Index k = 0; k < size(); ++k) s += std::pow(std::abs(lin(k)), (Scalar)P);
    return std::pow(s, (Scalar)1 / (Scalar)P);
  }
  Scalar maxCoeff() const {
    Scalar s = lin(0);
    for (Index k = 1; k < size(); ++k) s = std::max(s, lin(k));
    return s;
  }
  Scalar minCoeff() const {
    Scalar s = lin(0);
    for (Index k = 1; k < size(); ++k) s = std::min(s, lin(k));
    return s;
  }
  Scalar mean() const { return sum() / (Scalar)size(); }
  Scalar trace() const {
    Scalar s = 0;
    for (Index k = 0; k < std::min(rows(), cols()); ++k) s += derived().coeff(k, k);
    return s;
  }
  template <typename O>
  Scalar dot(const DenseBase<O>& o) const {
    if (o.size() != size()) throw std::logic_error("eigen shim: dot of vectors of different sizes");
    Scalar s = 0;
    for (Index k = 0; k < size(); ++k) s += lin(k) * o.lin(k);
    return s;
  }
  template <typename O>
  Matrix<Scalar, 3, 1> cross(const DenseBase<O>& o) const;
  template <typename O>
  PlainObject cwiseProduct(const DenseBase<O>& o) const;
  template <typename O>
  PlainObject cwiseQuotient(const DenseBase<O>& o) const;
  PlainObject cwiseAbs() const;
  PlainObject normalized() const;
  PlainObject eval() const { return PlainObject(derived()); }
  Matrix<Scalar, ColsAtCompileTime, RowsAtCompileTime> transpose() const;
  DiagonalWrapper<Scalar> asDiagonal() const;
};

// ---------------------------------------------------------------------------------- Matrix
template <typename S, int R, int C>
class Matrix : public DenseBase<Matrix<S, R, C>> {
 public:
  typedef S Scalar;
  static constexpr bool kFixed = R != Dynamic && C != Dynamic;
  typedef typename std::conditional<kFixed, std::array<S, (kFixed ? R * C : 1)>, std::vector<S>>::type Store;

  Matrix() : r_(R == Dynamic ? 0 : R), c_(C == Dynamic ? 0 : C) { init_store(); }
  // one size argument: a dynamic vector of that length
  explicit Matrix(Index n) : r_(R == 1 ? 1 : (R == Dynamic ? n : R)), c_(R == 1 ? (C == Dynamic ? n : C) : (C == Dynamic ? 1 : C)) {
    init_store();
  }
  Matrix(Index rows, Index cols) : r_(rows), c_(cols) { init_store(); }
  // three coefficients of a fixed 3-vector (Vector3d(x, y, z))
  Matrix(const S& x, const S& y, const S& z) : r_(3), c_(1) {
    init_store();
    d_[0] = x;
    d_[1] = y;
    d_[2] = z;
  }
  Matrix(const Matrix& o) = default;
  Matrix& operator=(const Matrix& o) = default;
  template <typename O>
  Matrix(const DenseBase<O>& o) : r_(R == Dynamic ? 0 : R), c_(C == Dynamic ? 0 : C) {
    init_store();
    assign(o);
  }
  Matrix(const DiagonalWrapper<S>& d) : r_(R == Dynamic ? 0 : R), c_(C == Dynamic ? 0 : C) {
    init_store();
    assign_diag(d);
  }
  template <typename O>
  Matrix& operator=(const DenseBase<O>& o) {
    assign(o);
    return *this;
  }
  Matrix& operator=(const DiagonalWrapper<S>& d) {
    assign_diag(d);
    return *this;
  }

  Index rows() const { return r_; }
  Index cols() const { return c_; }
  Index size() const { return r_ * c_; }
  S* data() { return d_.data(); }
  const S* data() const { return d_.data(); }
  S coeff(Index i, Index j) const { return d_[i + j * r_]; }
  S& operator()(Index i, Index j) { return d_[i + j * r_]; }
  const S& operator()(Index i, Index j) const { return d_[i + j * r_]; }
  S& operator()(Index k) { return d_[k]; }
  const S& operator()(Index k) const { return d_[k]; }
  S& operator[](Index k) { return d_[k]; }
  const S& operator[](Index k) const { return d_[k]; }
  S& x() { return d_[0]; }
  S& y() { return d_[1]; }
  S& z() { return d_[2]; }
  const S& x() const { return d_[0]; }
  const S& y() const { return d_[1]; }
  const S& z() const { return d_[2]; }

  void resize(Index n) {
    if (R == 1) resize(1, n);
    else resize(n, 1);
  }
  void resize(Index rows, Index cols) {
    if (kFixed) {  // fixed sizes keep their dimensions
      if (rows != R || cols != C) throw std::logic_error("eigen shim: resize of a fixed-size matrix");
      return;
    }
    r_ = rows;
    c_ = cols;
    init_store();
  }
  void conservativeResize(Index n) {
    Store old = d_;
    const Index on = size();
    resize(n);
    for (Index k = 0; k < std::min(on, n); ++k) d_[k] = old[k];
  }
  Matrix& setZero() { return setConstant(S(0)); }
  Matrix& setOnes() { return setConstant(S(1)); }
  Matrix& setConstant(const S& v) {
    std::fill(d_.begin(), d_.end(), v);
    return *this;
  }
  Matrix& setZero(Index n) {
    resize(n);
    return setZero();
  }
  Matrix& setZero(Index rows, Index cols) {
    resize(rows, cols);
    return setZero();
  }
  Matrix& setConstant(Index n, const S& v) {
    resize(n);
    return setConstant(v);
  }
  Matrix& setIdentity() {
    setZero();
    for (Index k = 0; k < std::min(r_, c_); ++k) (*this)(k, k) = S(1);
    return *this;
  }
  Matrix& setIdentity(Index rows, Index cols) {
    resize(rows, cols);
    return setIdentity();
  }
  Matrix& noalias() { return *this; }
  void normalize() { *this /= this->norm(); }

  static Matrix Zero() { return Matrix().setZero(); }
  static Matrix Zero(Index n) { return Matrix(n).setZero(); }
  static Matrix Zero(Index rows, Index cols) { return Matrix(rows, cols).setZero(); }
  static Matrix Ones() { return Matrix().setOnes(); }
  static Matrix Ones(Index n) { return Matrix(n).setOnes(); }
  static Matrix Ones(Index rows, Index cols) { return Matrix(rows, cols).setOnes(); }
  static Matrix Constant(const S& v) { return Matrix().setConstant(v); }
  static Matrix Constant(Index n, const S& v) { return Matrix(n).setConstant(v); }
  static Matrix Constant(Index rows, Index cols, const S& v) { return Matrix(rows, cols).setConstant(v); }
  static Matrix Identity() { return Matrix().setIdentity(); }
  static Matrix Identity(Index rows, Index cols) { return Matrix(rows, cols).setIdentity(); }
  static Matrix UnitX() { Matrix m = Zero(); m[0] = 1; return m; }
  static Matrix UnitY() { Matrix m = Zero(); m[1] = 1; return m; }
  static Matrix UnitZ() { Matrix m = Zero(); m[2] = 1; return m; }

  Block<Matrix, true> row(Index i) { return Block<Matrix, true>(this, i); }
  Block<Matrix, false> col(Index j) { return Block<Matrix, false>(this, j); }
  Block<const Matrix, true> row(Index i) const { return Block<const Matrix, true>(this, i); }
  Block<const Matrix, false> col(Index j) const { return Block<const Matrix, false>(this, j); }

  template <typename O>
  Matrix& operator+=(const DenseBase<O>& o) {
    check_same(o);
    for (Index k = 0; k < size(); ++k) d_[k] += o.lin(k);
    return *this;
  }
  template <typename O>
  Matrix& operator-=(const DenseBase<O>& o) {
    check_same(o);
    for (Index k = 0; k < size(); ++k) d_[k] -= o.lin(k);
    return *this;
  }
  template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
  Matrix& operator*=(const T& s) {
    for (auto& v : d_) v *= S(s);
    return *this;
  }
  template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
  Matrix& operator/=(const T& s) {
    for (auto& v : d_) v /= S(s);
    return *this;
  }

  // comma initializer: m << a, b, c; fills row by row (a vector in order)
  struct CommaInit {
    Matrix* m;
    Index k;
    CommaInit& operator,(const S& v) {
      m->set_row_major(k++, v);
      return *this;
    }
  };
  CommaInit operator<<(const S& v) {
    set_row_major(0, v);
    return CommaInit{this, 1};
  }
  void set_row_major(Index k, const S& v) { (*this)(k / c_, k % c_) = v; }
  // 3x3 determinant: expansion along row 0
  S determinant() const {
    if (r_ != 3 || c_ != 3) throw std::logic_error("eigen shim: determinant is implemented for 3x3 matrices");
    const Matrix& m = *this;
    return m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) - m(0, 1) * (m(1, 0) * m(2, 2) - m(1, 2) * m(2, 0)) +
           m(0, 2) * (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0));
  }
  // 3x3 inverse: cofactors, determinant from the cofactors of column 0, times 1/det
  Matrix inverse() const {
    if (r_ != 3 || c_ != 3) throw std::logic_error("eigen shim: inverse is implemented for 3x3 matrices");
    const Matrix& m = *this;
    auto cof = [&](int i, int j) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      return m(i1, j1) * m(i2, j2) - m(i1, j2) * m(i2, j1);
    };
    const S c0[3] = {cof(0, 0), cof(1, 0), cof(2, 0)};
    const S det = (c0[0] * m(0, 0) + c0[1] * m(1, 0)) + c0[2] * m(2, 0);
    const S id = S(1) / det;
    // r(i, j) = cofactor (j, i) / det; row 0 takes the column-0 cofactors
    Matrix r(3, 3);
    for (int j = 0; j < 3; ++j) r(0, j) = c0[j] * id;
    for (int i = 1; i < 3; ++i)
      for (int j = 0; j < 3; ++j) r(i, j) = cof(j, i) * id;
    return r;
  }
  // comparisons used by callers on small fixed vectors
  bool operator==(const Matrix& o) const { return r_ == o.r_ && c_ == o.c_ && std::equal(d_.begin(), d_.end(), o.d_.begin()); }
  bool operator!=(const Matrix& o) const { return !(*this == o); }

 private:
  void init_store() {
    if constexpr (kFixed) {
      d_.fill(S(0));
    } else {
      d_.assign((size_t)(r_ * c_), S(0));
    }
  }
  template <typename O>
  void check_same(const DenseBase<O>& o) const {
    if (o.size() != size()) throw std::logic_error("eigen shim: size mismatch");
  }
  template <typename O>
  void assign(const DenseBase<O>& o) {
    const Index orr = o.rows(), occ = o.cols();
    const bool vec_self = (R == 1 || C == 1), vec_o = (orr == 1 || occ == 1);
    if (vec_self && vec_o) {
      // vectors: row and column vectors convert into each other
      const Index n = orr * occ;
      if (R == 1) resize(1, n);
      else if (C == 1) resize(n, 1);
      Store tmp = make_store(n);
      for (Index k = 0; k < n; ++k) tmp[k] = o.lin(k);
      d_ = tmp;
      return;
    }
    Store tmp = make_store(orr * occ);
    for (Index j = 0; j < occ; ++j)
      for (Index i = 0; i < orr; ++i) tmp[i + j * orr] = o.derived().coeff(i, j);
    if (!kFixed) {
      r_ = orr;
      c_ = occ;
    } else if (orr != R || occ != C) {
      throw std::logic_error("eigen shim: assignment of a matrix of another shape");
    }
    d_ = tmp;
  }
  void assign_diag(const DiagonalWrapper<S>& d);
  Store make_store(Index n) const {
    Store s{};
    if constexpr (!kFixed) s.assign((size_t)n, S(0));
    return s;
  }
  Index r_, c_;
  Store d_;
};

// ---------------------------------------------------------------------------------- Block
// A row (IsRow) or column of a matrix, by reference.
template <typename M, bool IsRow>
class Block : public DenseBase<Block<M, IsRow>> {
 public:
  typedef typename traits<Block>::Scalar Scalar;
  Block(M* m, Index k) : m_(m), k_(k) {}
  Index rows() const { return IsRow ? 1 : m_->rows(); }
  Index cols() const { return IsRow ? m_->cols() : 1; }
  Index size() const { return IsRow ? m_->cols() : m_->rows(); }
  Scalar coeff(Index i, Index j) const { return IsRow ? (*m_)(k_, j) : (*m_)(i, k_); }
  Scalar operator()(Index k) const { return IsRow ? (*m_)(k_, k) : (*m_)(k, k_); }
  Scalar operator[](Index k) const { return (*this)(k); }
  Scalar& ref(Index k) { return IsRow ? (*m_)(k_, k) : (*m_)(k, k_); }
  Block& operator=(const Block& o) {
    Matrix<Scalar, Dynamic, 1> tmp(o.size());
    for (Index k = 0; k < o.size(); ++k) tmp[k] = o.lin(k);
    for (Index k = 0; k < size(); ++k) ref(k) = tmp[k];
    return *this;
  }
  template <typename O>
  Block& operator=(const DenseBase<O>& o) {
    if (o.size() != size()) throw std::logic_error("eigen shim: block assignment size mismatch");
    Matrix<Scalar, Dynamic, 1> tmp(o.size());
    for (Index k = 0; k < o.size(); ++k) tmp[k] = o.lin(k);
    for (Index k = 0; k < size(); ++k) ref(k) = tmp[k];
    return *this;
  }
  template <typename O>
  Block& operator+=(const DenseBase<O>& o) {
    for (Index k = 0; k < size(); ++k) ref(k) += o.lin(k);
    return *this;
  }
  template <typename O>
  Block& operator-=(const DenseBase<O>& o) {
    for (Index k = 0; k < size(); ++k) ref(k) -= o.lin(k);
    return *this;
  }
  template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
  Block& operator*=(const T& s) {
    for (Index k = 0; k < size(); ++k) ref(k) *= Scalar(s);
    return *this;
  }
  template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
  Block& operator/=(const T& s) {
    for (Index k = 0; k < size(); ++k) ref(k) /= Scalar(s);
    return *this;
  }

 private:
  M* m_;
  Index k_;
};

// ---------------------------------------------------------------------------------- diagonal
template <typename S>
class DiagonalWrapper {
 public:
  explicit DiagonalWrapper(std::vector<S> d) : d_(std::move(d)) {}
  Index rows() const { return (Index)d_.size(); }
  Index cols() const { return (Index)d_.size(); }
  const S& diag(Index k) const { return d_[k]; }

 private:
  std::vector<S> d_;
};

template <typename S, int R, int C>
void Matrix<S, R, C>::assign_diag(const DiagonalWrapper<S>& d) {
  const Index n = d.rows();
  if (!kFixed) {
    r_ = n;
    c_ = n;
    init_store();
  } else {
    setZero();
  }
  for (Index k = 0; k < n; ++k) (*this)(k, k) = d.diag(k);
}

// ---------------------------------------------------------------------------------- members of DenseBase
template <typename D>
template <typename O>
Matrix<typename DenseBase<D>::Scalar, 3, 1> DenseBase<D>::cross(const DenseBase<O>& o) const {
  Matrix<Scalar, 3, 1> r;
  r[0] = lin(1) * o.lin(2) - lin(2) * o.lin(1);
  r[1] = lin(2) * o.lin(0) - lin(0) * o.lin(2);
  r[2] = lin(0) * o.lin(1) - lin(1) * o.lin(0);
  return r;
}
template <typename D>
template <typename O>
typename DenseBase<D>::PlainObject DenseBase<D>::cwiseProduct(const DenseBase<O>& o) const {
  PlainObject r(derived());
  for (Index k = 0; k < size(); ++k) r(k) = lin(k) * o.lin(k);
  return r;
}
template <typename D>
template <typename O>
typename DenseBase<D>::PlainObject DenseBase<D>::cwiseQuotient(const DenseBase<O>& o) const {
  PlainObject r(derived());
  for (Index k = 0; k < size(); ++k) r(k) = lin(k) / o.lin(k);
  return r;
}
template <typename D>
typename DenseBase<D>::PlainObject DenseBase<D>::cwiseAbs() const {
  PlainObject r(derived());
  for (Index k = 0; k < size(); ++k) r(k) = std::abs(lin(k));
  return r;
}
template <typename D>
typename DenseBase<D>::PlainObject DenseBase<D>::normalized() const {
  PlainObject r(derived());
  const Scalar n = norm();
  for (Index k = 0; k < size(); ++k) r(k) = lin(k) / n;
  return r;
}
template <typename D>
Matrix<typename DenseBase<D>::Scalar, DenseBase<D>::ColsAtCompileTime, DenseBase<D>::RowsAtCompileTime> DenseBase<D>::transpose() const {
  Matrix<Scalar, ColsAtCompileTime, RowsAtCompileTime> r(cols(), rows());
  for (Index i = 0; i < rows(); ++i)
    for (Index j = 0; j < cols(); ++j) r(j, i) = derived().coeff(i, j);
  return r;
}
template <typename D>
DiagonalWrapper<typename DenseBase<D>::Scalar> DenseBase<D>::asDiagonal() const {
  std::vector<Scalar> v((size_t)size());
  for (Index k = 0; k < size(); ++k) v[k] = lin(k);
  return DiagonalWrapper<Scalar>(std::move(v));
}

// ---------------------------------------------------------------------------------- operators
template <typename A, typename B>
using SumResult = Matrix<typename traits<A>::Scalar, pick_dim(traits<A>::Rows, traits<B>::Rows), pick_dim(traits<A>::Cols, traits<B>::Cols)>;

template <typename A, typename B>
SumResult<A, B> operator+(const DenseBase<A>& a, const DenseBase<B>& b) {
  SumResult<A, B> r(a.derived());
  for (Index k = 0; k < r.size(); ++k) r(k) = a.lin(k) + b.lin(k);
  return r;
}
template <typename A, typename B>
SumResult<A, B> operator-(const DenseBase<A>& a, const DenseBase<B>& b) {
  SumResult<A, B> r(a.derived());
  for (Index k = 0; k < r.size(); ++k) r(k) = a.lin(k) - b.lin(k);
  return r;
}
template <typename A>
typename DenseBase<A>::PlainObject operator-(const DenseBase<A>& a) {
  typename DenseBase<A>::PlainObject r(a.derived());
  for (Index k = 0; k < r.size(); ++k) r(k) = -a.lin(k);
  return r;
}
template <typename T, typename A, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
typename DenseBase<A>::PlainObject operator*(const T& s, const DenseBase<A>& a) {
  typedef typename traits<A>::Scalar S;
  typename DenseBase<A>::PlainObject r(a.derived());
  for (Index k = 0; k < r.size(); ++k) r(k) = S(s) * a.lin(k);
  return r;
}
template <typename T, typename A, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
typename DenseBase<A>::PlainObject operator*(const DenseBase<A>& a, const T& s) {
  typedef typename traits<A>::Scalar S;
  typename DenseBase<A>::PlainObject r(a.derived());
  for (Index k = 0; k < r.size(); ++k) r(k) = a.lin(k) * S(s);
  return r;
}
template <typename T, typename A, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
typename DenseBase<A>::PlainObject operator/(const DenseBase<A>& a, const T& s) {
  typedef typename traits<A>::Scalar S;
  typename DenseBase<A>::PlainObject r(a.derived());
  for (Index k = 0; k < r.size(); ++k) r(k) = a.lin(k) / S(s);
  return r;
}
// matrix product, sums over the inner index in increasing order
template <typename A, typename B>
Matrix<typename traits<A>::Scalar, traits<A>::Rows, traits<B>::Cols> operator*(const DenseBase<A>& a, const DenseBase<B>& b) {
  typedef typename traits<A>::Scalar S;
  if (a.cols() != b.rows()) throw std::logic_error("eigen shim: product of matrices of incompatible shapes");
  Matrix<S, traits<A>::Rows, traits<B>::Cols> r(a.rows(), b.cols());
  for (Index j = 0; j < b.cols(); ++j)
    for (Index i = 0; i < a.rows(); ++i) {
      S s = 0;
      for (Index k = 0; k < a.cols(); ++k) s += a.derived().coeff(i, k) * b.derived().coeff(k, j);
      r(i, j) = s;
    }
  return r;
}
template <typename A>
Matrix<typename traits<A>::Scalar, traits<A>::Rows, Dynamic> operator*(const DenseBase<A>& a, const DiagonalWrapper<typename traits<A>::Scalar>& d) {
  typedef typename traits<A>::Scalar S;
  if (a.cols() != d.rows()) throw std::logic_error("eigen shim: matrix times diagonal of another size");
  Matrix<S, traits<A>::Rows, Dynamic> r(a.rows(), a.cols());
  for (Index j = 0; j < a.cols(); ++j)
    for (Index i = 0; i < a.rows(); ++i) r(i, j) = a.derived().coeff(i, j) * d.diag(j);
  return r;
}
template <typename B>
Matrix<typename traits<B>::Scalar, Dynamic, traits<B>::Cols> operator*(const DiagonalWrapper<typename traits<B>::Scalar>& d, const DenseBase<B>& b) {
  typedef typename traits<B>::Scalar S;
  if (b.rows() != d.rows()) throw std::logic_error("eigen shim: diagonal times matrix of another size");
  Matrix<S, Dynamic, traits<B>::Cols> r(b.rows(), b.cols());
  for (Index j = 0; j < b.cols(); ++j)
    for (Index i = 0; i < b.rows(); ++i) r(i, j) = d.diag(i) * b.derived().coeff(i, j);
  return r;
}

template <typename A>
std::ostream& operator<<(std::ostream& out, const DenseBase<A>& a) {
  for (Index i = 0; i < a.rows(); ++i) {
    for (Index j = 0; j < a.cols(); ++j) {
      if (j) out << " ";
      out << a.derived().coeff(i, j);
    }
    if (i + 1 < a.rows()) out << "\n";
  }
  return out;
}

// ---------------------------------------------------------------------------------- 3x3 algebra
// determinant and inverse of a fixed 3x3 matrix by cofactors
template <typename S>
S det3(const Matrix<S, 3, 3>& m) {
  return m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) - m(0, 1) * (m(1, 0) * m(2, 2) - m(1, 2) * m(2, 0)) +
         m(0, 2) * (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0));
}

typedef Matrix<double, 3, 1> Vector3d;
typedef Matrix<float, 3, 1> Vector3f;
typedef Matrix<int, 3, 1> Vector3i;
typedef Matrix<double, 2, 1> Vector2d;
typedef Matrix<double, 4, 1> Vector4d;
typedef Matrix<double, 3, 3> Matrix3d;
typedef Matrix<double, 2, 2> Matrix2d;
typedef Matrix<double, Dynamic, 1> VectorXd;
typedef Matrix<int, Dynamic, 1> VectorXi;
typedef Matrix<double, 1, Dynamic> RowVectorXd;
typedef Matrix<double, Dynamic, Dynamic> MatrixXd;
typedef Matrix<float, Dynamic, Dynamic> MatrixXf;

}  // namespace Eigen
