// Test-only stand-in for the parts of gismo's linear algebra (and of Eigen behind it) that the
// gsStructuralAnalysis solver headers use.  It exists so that those headers can be compiled
// UNCHANGED from the reference tree and run as a CPU oracle: it is never part of the product.
//
// Design: eager dense arithmetic in FP64 (the oracle's problems have a few hundred dofs).
//   * gsMatrix<T>: column-major dense matrix; gsVector<T>: one column.  Every operator returns a
//     new object (Eigen evaluates lazily; the values are the same up to the order of rounding).
//   * gsSparseMatrix<T>: a dense matrix behind the sparse interface the solvers call.
//   * gsSparseSolver<T>::get(name): "SimplicialLDLT" (LDL^T without pivoting, as Eigen's
//     simplicial factorisation; D exposed by vectorD()), "CGDiagonal" (Jacobi-preconditioned
//     conjugate gradients with Eigen's defaults: tolerance = machine epsilon, at most 2n
//     iterations, zero start), "SimplicialLLT", "SparseLU" (dense partial-pivoting LU).
//   * gsEigen::SelfAdjointEigenSolver / GeneralizedSelfAdjointEigenSolver: cyclic Jacobi
//     rotations, ascending eigenvalues, orthonormal (resp. B-normalised) eigenvectors.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <iomanip>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
// The reference calls abs() unqualified on floating-point values inside namespace gismo
// (gsALMBase.hpp:496-497 and 808-811, gsALMCrisfield.hpp:85 and 281).  With <cstdlib> alone the
// only global abs is C's int abs(int), and |x| is truncated to an integer.  The C++ wrappers
// <stdlib.h> and <math.h> put std::abs's floating-point overloads in the global namespace, as a
// translation unit that includes either of them anywhere gets them; that is the abs meant.
#include <math.h>
#include <stdlib.h>
#include <memory>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace gsEigen {
enum ComputationInfo { Success = 0, NumericalIssue = 1, NoConvergence = 2, InvalidInput = 3 };
}

namespace gismo {

typedef int index_t;
typedef double real_t;

namespace shim {
struct NullBuf : std::streambuf {
    int overflow(int c) override { return c; }
};
inline std::ostream& info() {
    static NullBuf nb;
    static std::ostream null(&nb);
    static const bool on = std::getenv("KLSA_REF_VERBOSE") != nullptr;
    return on ? std::cout : null;
}
}  // namespace shim

#define gsInfo ::gismo::shim::info()
#define gsWarn ::gismo::shim::info()
#define gsDebug ::gismo::shim::info()
#define gsDebugVar(x) ((void)0)
#define GISMO_STRINGIFY_(x) #x
#define GISMO_HPP_HEADER(x) GISMO_STRINGIFY_(x)
#define GISMO_ERROR(msg)                                                   \
    do {                                                                   \
        std::ostringstream gs_os_; gs_os_ << msg; throw std::runtime_error(gs_os_.str()); \
    } while (0)
#define GISMO_ASSERT(cond, msg) \
    do {                         \
        if (!(cond)) {           \
            std::ostringstream gs_os_; gs_os_ << msg; throw std::runtime_error(gs_os_.str()); \
        }                        \
    } while (0)
#define GISMO_ENSURE(cond, msg) GISMO_ASSERT(cond, msg)
#define GISMO_UNUSED(x) ((void)(x))
#define GISMO_NO_IMPLEMENTATION GISMO_ERROR("not implemented in the test shim");

namespace math {
using std::abs;
using std::sqrt;
using std::pow;
using std::exp;
using std::log;
using std::log10;
using std::min;
using std::max;
using std::floor;
using std::ceil;
template <class T> inline T sign(T v) { return (T(0) < v) - (v < T(0)); }
template <class T> inline bool isinf(T v) { return std::isinf(v); }
template <class T> inline bool isnan(T v) { return std::isnan(v); }
}  // namespace math

template <class T = real_t> class gsMatrix;
template <class T = real_t> class gsVector;
template <class T = real_t> class gsSparseMatrix;
template <class T> struct gsRowBlock;

// Reference to a matrix's coefficients as an array (m.array() += s, m.array().abs()).
template <class T>
struct gsArrayRef {
    gsMatrix<T>& m;
    gsArrayRef& operator+=(T s) { for (auto& v : m.d) v += s; return *this; }
    gsArrayRef& operator-=(T s) { for (auto& v : m.d) v -= s; return *this; }
    gsArrayRef& operator*=(T s) { for (auto& v : m.d) v *= s; return *this; }
    gsMatrix<T> abs() const { gsMatrix<T> r = m; for (auto& v : r.d) v = std::abs(v); return r; }
};

template <class T>
struct gsColwise {
    const gsMatrix<T>& m;
    gsMatrix<T> minCoeff() const;
    gsMatrix<T> maxCoeff() const;
};

template <class T>
class gsMatrix {
public:
    typedef T Scalar;
    typedef gsMatrix Base;
    typedef std::unique_ptr<gsMatrix> uPtr;
    index_t r = 0, c = 0;
    std::vector<T> d;

    gsMatrix() {}
    gsMatrix(index_t rows, index_t cols) : r(rows), c(cols), d((size_t)rows * cols, T(0)) {}
    virtual ~gsMatrix() {}

    index_t rows() const { return r; }
    index_t cols() const { return c; }
    index_t size() const { return r * c; }
    T* data() { return d.data(); }
    const T* data() const { return d.data(); }

    T& operator()(index_t i, index_t j) { return d[(size_t)j * r + i]; }
    const T& operator()(index_t i, index_t j) const { return d[(size_t)j * r + i]; }
    T& operator()(index_t i) { return d[i]; }
    const T& operator()(index_t i) const { return d[i]; }
    T& operator[](index_t i) { return d[i]; }
    const T& operator[](index_t i) const { return d[i]; }
    T& at(index_t i) { return d.at(i); }
    const T& at(index_t i) const { return d.at(i); }
    T value() const { GISMO_ASSERT(r * c == 1, "value() of a non-1x1 matrix"); return d[0]; }

    void resize(index_t rows, index_t cols) { r = rows; c = cols; d.assign((size_t)rows * cols, T(0)); }
    gsMatrix& setZero() { std::fill(d.begin(), d.end(), T(0)); return *this; }
    gsMatrix& setZero(index_t rows, index_t cols) { resize(rows, cols); return *this; }
    gsMatrix& setOnes() { std::fill(d.begin(), d.end(), T(1)); return *this; }
    gsMatrix& setConstant(T v) { std::fill(d.begin(), d.end(), v); return *this; }
    gsMatrix& setIdentity() { setZero(); for (index_t i = 0; i < std::min(r, c); ++i) (*this)(i, i) = T(1); return *this; }

    static gsMatrix Zero(index_t rows, index_t cols) { return gsMatrix(rows, cols); }
    static gsMatrix Ones(index_t rows, index_t cols) { gsMatrix m(rows, cols); m.setOnes(); return m; }
    static gsMatrix Identity(index_t rows, index_t cols) { gsMatrix m(rows, cols); m.setIdentity(); return m; }

    T squaredNorm() const { T s = 0; for (T v : d) s += v * v; return s; }
    T norm() const { return std::sqrt(squaredNorm()); }
    void normalize() { const T n = norm(); if (n > 0) for (auto& v : d) v /= n; }
    gsMatrix normalized() const { gsMatrix m = *this; m.normalize(); return m; }
    T dot(const gsMatrix& o) const {
        GISMO_ASSERT(size() == o.size(), "dot: size mismatch " << size() << " vs " << o.size());
        T s = 0;
        for (size_t i = 0; i < d.size(); ++i) s += d[i] * o.d[i];
        return s;
    }
    T sum() const { T s = 0; for (T v : d) s += v; return s; }
    T minCoeff() const { return *std::min_element(d.begin(), d.end()); }
    T maxCoeff() const { return *std::max_element(d.begin(), d.end()); }
    gsMatrix transpose() const {
        gsMatrix t(c, r);
        for (index_t j = 0; j < c; ++j)
            for (index_t i = 0; i < r; ++i) t(j, i) = (*this)(i, j);
        return t;
    }
    gsVector<T> col(index_t j) const;
    gsMatrix row(index_t i) const { gsMatrix m(1, c); for (index_t j = 0; j < c; ++j) m(0, j) = (*this)(i, j); return m; }
    gsColwise<T> colwise() const { return gsColwise<T>{*this}; }
    gsArrayRef<T> array() { return gsArrayRef<T>{*this}; }
    gsMatrix toDense() const { return *this; }
    gsSparseMatrix<T> sparseView() const;
    // rows [0, n) / [rows - n, rows) as an assignable block (Eigen's topRows / bottomRows)
    gsRowBlock<T> topRows(index_t n) { return gsRowBlock<T>{*this, 0, n}; }
    gsRowBlock<T> bottomRows(index_t n) { return gsRowBlock<T>{*this, r - n, n}; }
    gsMatrix inverse() const;

    gsMatrix& operator+=(const gsMatrix& o) { check_same(o); for (size_t i = 0; i < d.size(); ++i) d[i] += o.d[i]; return *this; }
    gsMatrix& operator-=(const gsMatrix& o) { check_same(o); for (size_t i = 0; i < d.size(); ++i) d[i] -= o.d[i]; return *this; }
    gsMatrix& operator*=(T s) { for (auto& v : d) v *= s; return *this; }
    gsMatrix& operator/=(T s) { for (auto& v : d) v /= s; return *this; }

    friend gsMatrix operator+(const gsMatrix& a, const gsMatrix& b) { gsMatrix m = a; m += b; return m; }
    friend gsMatrix operator-(const gsMatrix& a, const gsMatrix& b) { gsMatrix m = a; m -= b; return m; }
    friend gsMatrix operator-(const gsMatrix& a) { gsMatrix m = a; for (auto& v : m.d) v = -v; return m; }
    friend gsMatrix operator*(const gsMatrix& a, const T& s) { gsMatrix m = a; m *= s; return m; }
    friend gsMatrix operator*(const T& s, const gsMatrix& a) { gsMatrix m = a; m *= s; return m; }
    friend gsMatrix operator/(const gsMatrix& a, const T& s) { gsMatrix m = a; m /= s; return m; }
    // a 1x1 product used as a scalar divisor, as Eigen allows for inner products
    friend gsMatrix operator/(const gsMatrix& a, const gsMatrix& s) { return a / s.value(); }
    friend gsMatrix operator*(const gsMatrix& a, const gsMatrix& b) {
        GISMO_ASSERT(a.c == b.r, "product: inner dimensions " << a.c << " vs " << b.r);
        gsMatrix m(a.r, b.c);
        for (index_t j = 0; j < b.c; ++j)
            for (index_t k = 0; k < a.c; ++k) {
                const T bkj = b(k, j);
                if (bkj == T(0)) continue;
                for (index_t i = 0; i < a.r; ++i) m(i, j) += a(i, k) * bkj;
            }
        return m;
    }
    friend std::ostream& operator<<(std::ostream& os, const gsMatrix& m) {
        for (index_t i = 0; i < m.r; ++i) {
            for (index_t j = 0; j < m.c; ++j) os << (j ? " " : "") << m(i, j);
            os << "\n";
        }
        return os;
    }

protected:
    void check_same(const gsMatrix& o) const {
        GISMO_ASSERT(r == o.r && c == o.c, "size mismatch " << r << "x" << c << " vs " << o.r << "x" << o.c);
    }
};

template <class T>
class gsVector : public gsMatrix<T> {
public:
    typedef std::unique_ptr<gsVector> uPtr;
    gsVector() : gsMatrix<T>(0, 1) {}
    explicit gsVector(index_t n) : gsMatrix<T>(n, 1) {}
    gsVector(const gsMatrix<T>& m) : gsMatrix<T>(m) {
        if (this->c != 1) {             // a row vector becomes a column
            GISMO_ASSERT(this->r == 1 || this->r * this->c == 0, "gsVector from a " << this->r << "x" << this->c << " matrix");
            this->r = this->r * this->c;
            this->c = 1;
        }
    }
    gsVector& operator=(const gsMatrix<T>& m) { *this = gsVector(m); return *this; }
    void resize(index_t n) { gsMatrix<T>::resize(n, 1); }
    void resize(index_t rows, index_t cols) { gsMatrix<T>::resize(rows, cols); }
    static gsVector Zero(index_t n) { return gsVector(n); }
    static gsVector Ones(index_t n) { gsVector v(n); v.setOnes(); return v; }
    static gsVector Constant(index_t n, T s) { gsVector v(n); v.setConstant(s); return v; }
    gsVector& setZero() { gsMatrix<T>::setZero(); return *this; }
    gsVector& setZero(index_t n) { resize(n); return *this; }
    gsVector& setOnes() { gsMatrix<T>::setOnes(); return *this; }
    gsVector& setOnes(index_t n) { resize(n); gsMatrix<T>::setOnes(); return *this; }
};

template <class T>
gsVector<T> gsMatrix<T>::col(index_t j) const {
    gsVector<T> v(r);
    for (index_t i = 0; i < r; ++i) v(i) = (*this)(i, j);
    return v;
}

template <class T>
gsMatrix<T> gsColwise<T>::minCoeff() const {
    gsMatrix<T> out(1, m.cols());
    for (index_t j = 0; j < m.cols(); ++j) {
        T v = std::numeric_limits<T>::infinity();
        for (index_t i = 0; i < m.rows(); ++i) v = std::min(v, m(i, j));
        out(0, j) = v;
    }
    return out;
}
template <class T>
gsMatrix<T> gsColwise<T>::maxCoeff() const {
    gsMatrix<T> out(1, m.cols());
    for (index_t j = 0; j < m.cols(); ++j) {
        T v = -std::numeric_limits<T>::infinity();
        for (index_t i = 0; i < m.rows(); ++i) v = std::max(v, m(i, j));
        out(0, j) = v;
    }
    return out;
}

// Dense LU with partial pivoting: factors a copy of A in place; returns false when singular.
template <class T>
bool lu_factor(gsMatrix<T>& A, std::vector<index_t>& piv) {
    const index_t n = A.rows();
    piv.resize(n);
    for (index_t k = 0; k < n; ++k) {
        index_t p = k;
        for (index_t i = k + 1; i < n; ++i)
            if (std::abs(A(i, k)) > std::abs(A(p, k))) p = i;
        piv[k] = p;
        if (A(p, k) == T(0)) return false;
        if (p != k)
            for (index_t j = 0; j < n; ++j) std::swap(A(k, j), A(p, j));
        for (index_t i = k + 1; i < n; ++i) {
            A(i, k) /= A(k, k);
            const T l = A(i, k);
            if (l != T(0))
                for (index_t j = k + 1; j < n; ++j) A(i, j) -= l * A(k, j);
        }
    }
    return true;
}
template <class T>
void lu_solve(const gsMatrix<T>& LU, const std::vector<index_t>& piv, T* b) {
    const index_t n = LU.rows();
    for (index_t k = 0; k < n; ++k) std::swap(b[k], b[piv[k]]);
    for (index_t i = 0; i < n; ++i)
        for (index_t k = 0; k < i; ++k) b[i] -= LU(i, k) * b[k];
    for (index_t i = n - 1; i >= 0; --i) {
        for (index_t k = i + 1; k < n; ++k) b[i] -= LU(i, k) * b[k];
        b[i] /= LU(i, i);
    }
}

template <class T>
gsMatrix<T> gsMatrix<T>::inverse() const {
    GISMO_ASSERT(r == c, "inverse of a non-square matrix");
    gsMatrix<T> LU = *this;
    std::vector<index_t> piv;
    if (!lu_factor(LU, piv)) throw std::runtime_error("inverse: singular matrix");
    gsMatrix<T> X = gsMatrix<T>::Identity(r, r);
    for (index_t j = 0; j < r; ++j) lu_solve(LU, piv, &X(0, j));
    return X;
}

// Sparse interface over dense storage.
template <class T>
class gsSparseMatrix : public gsMatrix<T> {
public:
    typedef std::unique_ptr<gsSparseMatrix> uPtr;
    gsSparseMatrix() {}
    gsSparseMatrix(index_t rows, index_t cols) : gsMatrix<T>(rows, cols) {}
    gsSparseMatrix(const gsMatrix<T>& m) : gsMatrix<T>(m) {}
    gsSparseMatrix& operator=(const gsMatrix<T>& m) { gsMatrix<T>::operator=(m); return *this; }
    gsMatrix<T> toDense() const { return *this; }
    index_t nonZeros() const { index_t k = 0; for (T v : this->d) k += v != T(0); return k; }
    T coeff(index_t i, index_t j) const { return (*this)(i, j); }
    T& coeffRef(index_t i, index_t j) { return (*this)(i, j); }
    void makeCompressed() {}
};

template <class T>
gsSparseMatrix<T> gsMatrix<T>::sparseView() const { return gsSparseMatrix<T>(*this); }

template <class T>
struct gsRowBlock {
    gsMatrix<T>& m;
    index_t r0, n;
    gsMatrix<T> value() const {
        gsMatrix<T> out(n, m.cols());
        for (index_t j = 0; j < m.cols(); ++j)
            for (index_t i = 0; i < n; ++i) out(i, j) = m(r0 + i, j);
        return out;
    }
    operator gsMatrix<T>() const { return value(); }
    friend gsMatrix<T> operator*(const T& s, const gsRowBlock& b) { return s * b.value(); }
    friend gsMatrix<T> operator*(const gsRowBlock& b, const T& s) { return b.value() * s; }
    friend gsMatrix<T> operator*(const gsMatrix<T>& a, const gsRowBlock& b) { return a * b.value(); }
    friend gsMatrix<T> operator+(const gsRowBlock& a, const gsMatrix<T>& b) { return a.value() + b; }
    friend gsMatrix<T> operator-(const gsRowBlock& a, const gsMatrix<T>& b) { return a.value() - b; }
    gsRowBlock& operator=(const gsMatrix<T>& b) {
        GISMO_ASSERT(b.rows() == n && b.cols() == m.cols(), "row block size");
        for (index_t j = 0; j < m.cols(); ++j)
            for (index_t i = 0; i < n; ++i) m(r0 + i, j) = b(i, j);
        return *this;
    }
    gsRowBlock& operator+=(const gsMatrix<T>& b) {
        GISMO_ASSERT(b.rows() == n && b.cols() == m.cols(), "row block size");
        for (index_t j = 0; j < m.cols(); ++j)
            for (index_t i = 0; i < n; ++i) m(r0 + i, j) += b(i, j);
        return *this;
    }
};

// ---- sparse solvers -------------------------------------------------------------------------
template <class T>
class gsSparseSolverBase {
public:
    virtual ~gsSparseSolverBase() {}
    virtual void compute(const gsMatrix<T>& A) = 0;
    virtual gsVector<T> solve(const gsMatrix<T>& b) const = 0;
    virtual gsEigen::ComputationInfo info() const { return m_info; }
    virtual std::string detail() const { return ""; }

protected:
    gsEigen::ComputationInfo m_info = gsEigen::Success;
};

template <class T = real_t>
struct gsSparseSolver {
    typedef gsSparseSolverBase<T> Base;
    typedef std::unique_ptr<Base> uPtr;

    // LDL^T without pivoting (Eigen's simplicial factorisation pivots nothing; a zero pivot
    // reports NumericalIssue).
    class SimplicialLDLT : public Base {
    public:
        void compute(const gsMatrix<T>& A) override {
            const index_t n = A.rows();
            L = gsMatrix<T>::Identity(n, n);
            D = gsVector<T>(n);
            this->m_info = gsEigen::Success;
            gsMatrix<T> W = A;                    // lower triangle used
            for (index_t j = 0; j < n; ++j) {
                T dj = W(j, j);
                for (index_t k = 0; k < j; ++k) dj -= L(j, k) * L(j, k) * D(k);
                D(j) = dj;
                if (dj == T(0)) {                 // Eigen checks for an exact zero only
                    this->m_info = gsEigen::NumericalIssue;
                    return;
                }
                for (index_t i = j + 1; i < n; ++i) {
                    T s = W(i, j);
                    for (index_t k = 0; k < j; ++k) s -= L(i, k) * L(j, k) * D(k);
                    L(i, j) = s / dj;
                }
            }
        }
        gsVector<T> solve(const gsMatrix<T>& b) const override {
            const index_t n = L.rows();
            gsVector<T> x(b);
            for (index_t i = 0; i < n; ++i)
                for (index_t k = 0; k < i; ++k) x(i) -= L(i, k) * x(k);
            for (index_t i = 0; i < n; ++i) x(i) /= D(i);
            for (index_t i = n - 1; i >= 0; --i)
                for (index_t k = i + 1; k < n; ++k) x(i) -= L(k, i) * x(k);
            return x;
        }
        gsVector<T> vectorD() const { return D; }

    private:
        gsMatrix<T> L;
        gsVector<T> D;
    };

    class SimplicialLLT : public Base {
    public:
        void compute(const gsMatrix<T>& A) override {
            const index_t n = A.rows();
            L = gsMatrix<T>(n, n);
            this->m_info = gsEigen::Success;
            for (index_t j = 0; j < n; ++j) {
                T s = A(j, j);
                for (index_t k = 0; k < j; ++k) s -= L(j, k) * L(j, k);
                if (!(s > T(0))) { this->m_info = gsEigen::NumericalIssue; return; }
                L(j, j) = std::sqrt(s);
                for (index_t i = j + 1; i < n; ++i) {
                    T t = A(i, j);
                    for (index_t k = 0; k < j; ++k) t -= L(i, k) * L(j, k);
                    L(i, j) = t / L(j, j);
                }
            }
        }
        gsVector<T> solve(const gsMatrix<T>& b) const override {
            const index_t n = L.rows();
            gsVector<T> x(b);
            for (index_t i = 0; i < n; ++i) {
                for (index_t k = 0; k < i; ++k) x(i) -= L(i, k) * x(k);
                x(i) /= L(i, i);
            }
            for (index_t i = n - 1; i >= 0; --i) {
                for (index_t k = i + 1; k < n; ++k) x(i) -= L(k, i) * x(k);
                x(i) /= L(i, i);
            }
            return x;
        }
        const gsMatrix<T>& matrixL() const { return L; }

    private:
        gsMatrix<T> L;
    };

    class SparseLU : public Base {
    public:
        SparseLU() {}
        explicit SparseLU(const gsMatrix<T>& A) { compute(A); }
        void compute(const gsMatrix<T>& A) override {
            LU = A;
            this->m_info = lu_factor(LU, piv) ? gsEigen::Success : gsEigen::NumericalIssue;
        }
        gsVector<T> solve(const gsMatrix<T>& b) const override {
            gsVector<T> x(b);
            lu_solve(LU, piv, x.data());
            return x;
        }
        // several right-hand sides (the columns of B), as Eigen's solve of a matrix
        gsMatrix<T> solve(const gsSparseMatrix<T>& B) const {
            gsMatrix<T> X(B);
            for (index_t j = 0; j < X.cols(); ++j) lu_solve(LU, piv, &X(0, j));
            return X;
        }

    private:
        gsMatrix<T> LU;
        std::vector<index_t> piv;
    };
    typedef SparseLU LU;

    // Eigen::ConjugateGradient with the DiagonalPreconditioner and its defaults: tolerance =
    // machine epsilon on ||r|| / ||b||, at most 2n iterations, start at zero.
    class CGDiagonal : public Base {
    public:
        void compute(const gsMatrix<T>& A_) override {
            A = A_;
            const index_t n = A.rows();
            inv = gsVector<T>(n);
            for (index_t i = 0; i < n; ++i) inv(i) = A(i, i) != T(0) ? T(1) / A(i, i) : T(1);
            this->m_info = gsEigen::Success;
        }
        gsVector<T> solve(const gsMatrix<T>& b_) const override {
            const index_t n = A.rows();
            gsVector<T> b(b_), x(n);
            const T bn2 = b.squaredNorm();
            if (bn2 == T(0)) return x;
            const T tol = std::numeric_limits<T>::epsilon();
            const T thr = tol * tol * bn2;
            gsVector<T> r = b, z(n), p(n);
            for (index_t i = 0; i < n; ++i) z(i) = inv(i) * r(i);
            p = z;
            T rz = r.dot(z);
            for (index_t it = 0; it < 2 * n; ++it) {
                gsVector<T> q = A * p;
                const T alpha = rz / p.dot(q);
                x += alpha * p;
                r -= alpha * q;
                if (r.squaredNorm() < thr) break;
                for (index_t i = 0; i < n; ++i) z(i) = inv(i) * r(i);
                const T rz1 = r.dot(z);
                p = z + (rz1 / rz) * p;
                rz = rz1;
            }
            return x;
        }

    private:
        gsMatrix<T> A;
        gsVector<T> inv;
    };

    static uPtr get(const std::string& name) {
        if (name == "SimplicialLDLT") return uPtr(new SimplicialLDLT());
        if (name == "SimplicialLLT") return uPtr(new SimplicialLLT());
        if (name == "CGDiagonal") return uPtr(new CGDiagonal());
        if (name == "SparseLU") return uPtr(new SparseLU());
        throw std::runtime_error("test shim: no sparse solver named " + name);
    }
};

// ---- dense symmetric eigensolvers ------------------------------------------------------------
namespace shim {
// Cyclic Jacobi method for a symmetric matrix (Jacobi 1846; the two-sided rotation as in Golub &
// Van Loan, Matrix Computations, section 8.5): sweeps of plane rotations, each annihilating one
// off-diagonal pair, until the off-diagonal mass is below eps^2 times the total.  A is
// overwritten (its diagonal converges to the eigenvalues), V accumulates the rotations.
template <class T>
bool jacobi_eigen(gsMatrix<T>& A, gsMatrix<T>& V) {
    const index_t n = A.rows();
    V = gsMatrix<T>::Identity(n, n);
    T total = 0;
    for (T v : A.d) total += v * v;
    const T eps = std::numeric_limits<T>::epsilon();
    for (int sweep = 0; sweep < 100; ++sweep) {
        T off = 0;
        for (index_t q = 0; q < n; ++q)
            for (index_t p = 0; p < q; ++p) off += 2 * A(p, q) * A(p, q);
        if (off <= eps * eps * total) return true;
        for (index_t q = 1; q < n; ++q)
            for (index_t p = 0; p < q; ++p) {
                const T apq = A(p, q);
                if (apq == T(0)) continue;
                // rotation [c s; -s c] that zeroes A(p,q): tan(2 theta) = 2 apq / (aqq - app)
                const T tau = (A(q, q) - A(p, p)) / (2 * apq);
                const T t = (tau >= 0 ? T(1) : T(-1)) / (std::abs(tau) + std::sqrt(T(1) + tau * tau));
                const T c = T(1) / std::sqrt(T(1) + t * t), s = t * c;
                for (index_t k = 0; k < n; ++k) {        // columns p, q
                    const T akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - s * akq;
                    A(k, q) = s * akp + c * akq;
                }
                for (index_t k = 0; k < n; ++k) {        // rows p, q
                    const T apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - s * aqk;
                    A(q, k) = s * apk + c * aqk;
                }
                A(p, q) = A(q, p) = 0;
                for (index_t k = 0; k < n; ++k) {
                    const T vkp = V(k, p), vkq = V(k, q);
                    V(k, p) = c * vkp - s * vkq;
                    V(k, q) = s * vkp + c * vkq;
                }
            }
    }
    return false;
}

// eigenvalues ascending, vectors permuted alike
template <class T>
void sort_pairs(std::vector<T>& dd, gsMatrix<T>& z) {
    const index_t n = (index_t)dd.size();
    std::vector<index_t> idx(n);
    for (index_t i = 0; i < n; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](index_t a, index_t b) { return dd[a] < dd[b]; });
    gsMatrix<T> z2(z.rows(), n);
    std::vector<T> d2(n);
    for (index_t j = 0; j < n; ++j) {
        d2[j] = dd[idx[j]];
        for (index_t i = 0; i < z.rows(); ++i) z2(i, j) = z(i, idx[j]);
    }
    dd = d2;
    z = z2;
}
}  // namespace shim

}  // namespace gismo

namespace gsEigen {
template <class M>
class SelfAdjointEigenSolver {
    typedef typename M::Scalar T;

public:
    SelfAdjointEigenSolver() {}
    explicit SelfAdjointEigenSolver(const gismo::gsMatrix<T>& A) { compute(A); }
    SelfAdjointEigenSolver& compute(const gismo::gsMatrix<T>& A) {
        gismo::gsMatrix<T> W = A, z;
        for (gismo::index_t j = 0; j < W.cols(); ++j)      // symmetric part (Eigen reads the lower triangle)
            for (gismo::index_t i = j + 1; i < W.rows(); ++i) W(j, i) = W(i, j);
        m_info = gismo::shim::jacobi_eigen(W, z) ? Success : NoConvergence;
        std::vector<T> dd((size_t)W.rows());
        for (gismo::index_t i = 0; i < W.rows(); ++i) dd[(size_t)i] = W(i, i);
        gismo::shim::sort_pairs(dd, z);
        m_values = gismo::gsVector<T>((gismo::index_t)dd.size());
        for (size_t i = 0; i < dd.size(); ++i) m_values((gismo::index_t)i) = dd[i];
        m_vectors = z;
        return *this;
    }
    const gismo::gsVector<T>& eigenvalues() const { return m_values; }
    const gismo::gsMatrix<T>& eigenvectors() const { return m_vectors; }
    ComputationInfo info() const { return m_info; }

protected:
    gismo::gsVector<T> m_values;
    gismo::gsMatrix<T> m_vectors;
    ComputationInfo m_info = Success;
};

// A x = lambda B x with B symmetric positive definite: B = L L^T, C = L^-1 A L^-T, C y =
// lambda y, x = L^-T y (so that x^T B x = 1).
template <class M>
class GeneralizedSelfAdjointEigenSolver : public SelfAdjointEigenSolver<M> {
    typedef typename M::Scalar T;
    typedef gismo::index_t I;

public:
    GeneralizedSelfAdjointEigenSolver() {}
    GeneralizedSelfAdjointEigenSolver& compute(const gismo::gsMatrix<T>& A, const gismo::gsMatrix<T>& B) {
        const I n = A.rows();
        typename gismo::gsSparseSolver<T>::SimplicialLLT llt;
        llt.compute(B);
        if (llt.info() != Success) throw std::runtime_error("generalized eigenproblem: B is not positive definite");
        const gismo::gsMatrix<T>& L = llt.matrixL();
        gismo::gsMatrix<T> C = A;
        for (I j = 0; j < n; ++j)                    // C <- L^-1 C
            for (I i = 0; i < n; ++i) {
                T s = C(i, j);
                for (I k = 0; k < i; ++k) s -= L(i, k) * C(k, j);
                C(i, j) = s / L(i, i);
            }
        for (I i = 0; i < n; ++i)                    // C <- C L^-T
            for (I j = 0; j < n; ++j) {
                T s = C(i, j);
                for (I k = 0; k < j; ++k) s -= C(i, k) * L(j, k);
                C(i, j) = s / L(j, j);
            }
        for (I j = 0; j < n; ++j)
            for (I i = j + 1; i < n; ++i) C(i, j) = C(j, i) = 0.5 * (C(i, j) + C(j, i));
        SelfAdjointEigenSolver<M>::compute(C);
        gismo::gsMatrix<T>& X = this->m_vectors;
        for (I j = 0; j < n; ++j)                    // X <- L^-T Y
            for (I i = n - 1; i >= 0; --i) {
                T s = X(i, j);
                for (I k = i + 1; k < n; ++k) s -= L(k, i) * X(k, j);
                X(i, j) = s / L(i, i);
            }
        return *this;
    }
};
}  // namespace gsEigen
