// Test-only stand-in for the linear operators and the GMRES solver of gismo's gsSolver module,
// as gsDynamicImplicitEuler uses them: an identity operator, a matrix operator, a 2x2 block
// operator, and gsGMRes::solve.  This project's own code.
//
// The stand-in's GMRES solves the operator EXACTLY: it forms the operator's dense matrix column
// by column (apply to the unit vectors) and solves it with the stand-in's pivoted LU.  That is
// the solution an unpreconditioned GMRES converges to, so the implicit-Euler step logic runs
// unchanged while its inner solve carries no iteration error.
#pragma once

#include <memory>
#include <vector>

#include <gsCore/gsLinearAlgebra.h>

namespace gismo {

template <class T = real_t>
class gsLinearOperator {
public:
    typedef std::shared_ptr<gsLinearOperator> Ptr;
    virtual ~gsLinearOperator() {}
    virtual void apply(const gsMatrix<T>& in, gsMatrix<T>& out) const = 0;
    virtual index_t rows() const = 0;
    virtual index_t cols() const = 0;
};

template <class T = real_t>
class gsIdentityOp : public gsLinearOperator<T> {
public:
    typedef std::shared_ptr<gsIdentityOp> Ptr;
    explicit gsIdentityOp(index_t n) : n_(n) {}
    static Ptr make(index_t n) { return Ptr(new gsIdentityOp(n)); }
    void apply(const gsMatrix<T>& in, gsMatrix<T>& out) const override { out = in; }
    index_t rows() const override { return n_; }
    index_t cols() const override { return n_; }

private:
    index_t n_;
};

template <class T = real_t>
class gsMatrixOp : public gsLinearOperator<T> {
public:
    typedef std::shared_ptr<gsMatrixOp> Ptr;
    explicit gsMatrixOp(const gsMatrix<T>& m) : m_(m) {}
    void apply(const gsMatrix<T>& in, gsMatrix<T>& out) const override { out = m_ * in; }
    index_t rows() const override { return m_.rows(); }
    index_t cols() const override { return m_.cols(); }

private:
    gsMatrix<T> m_;     // a copy, as gismo's makeMatrixOp of a temporary keeps one
};

template <class T>
typename gsMatrixOp<T>::Ptr makeMatrixOp(const gsMatrix<T>& m) {
    return typename gsMatrixOp<T>::Ptr(new gsMatrixOp<T>(m));
}

template <class T = real_t>
class gsBlockOp : public gsLinearOperator<T> {
public:
    typedef std::shared_ptr<gsBlockOp> Ptr;
    typedef typename gsLinearOperator<T>::Ptr BasePtr;
    gsBlockOp(index_t nr, index_t nc) : nr_(nr), nc_(nc), ops_((size_t)(nr * nc)) {}
    static Ptr make(index_t nr, index_t nc) { return Ptr(new gsBlockOp(nr, nc)); }
    void addOperator(index_t i, index_t j, const BasePtr& op) { ops_[(size_t)(i * nc_ + j)] = op; }

    index_t rows() const override {
        index_t s = 0;
        for (index_t i = 0; i < nr_; ++i) s += row_size(i);
        return s;
    }
    index_t cols() const override {
        index_t s = 0;
        for (index_t j = 0; j < nc_; ++j) s += col_size(j);
        return s;
    }
    void apply(const gsMatrix<T>& in, gsMatrix<T>& out) const override {
        out = gsMatrix<T>(rows(), in.cols());
        index_t r0 = 0;
        for (index_t i = 0; i < nr_; ++i) {
            index_t c0 = 0;
            for (index_t j = 0; j < nc_; ++j) {
                const BasePtr& op = ops_[(size_t)(i * nc_ + j)];
                if (op) {
                    gsMatrix<T> x(op->cols(), in.cols()), y;
                    for (index_t k = 0; k < in.cols(); ++k)
                        for (index_t a = 0; a < op->cols(); ++a) x(a, k) = in(c0 + a, k);
                    op->apply(x, y);
                    for (index_t k = 0; k < in.cols(); ++k)
                        for (index_t a = 0; a < op->rows(); ++a) out(r0 + a, k) += y(a, k);
                }
                c0 += col_size(j);
            }
            r0 += row_size(i);
        }
    }

private:
    index_t row_size(index_t i) const {
        for (index_t j = 0; j < nc_; ++j)
            if (ops_[(size_t)(i * nc_ + j)]) return ops_[(size_t)(i * nc_ + j)]->rows();
        return 0;
    }
    index_t col_size(index_t j) const {
        for (index_t i = 0; i < nr_; ++i)
            if (ops_[(size_t)(i * nc_ + j)]) return ops_[(size_t)(i * nc_ + j)]->cols();
        return 0;
    }
    index_t nr_, nc_;
    std::vector<BasePtr> ops_;
};

template <class T = real_t>
class gsGMRes {
public:
    typedef typename gsLinearOperator<T>::Ptr OpPtr;
    explicit gsGMRes(const OpPtr& op) : op_(op) {}
    // x = A^-1 b, exactly (see the file comment)
    void solve(const gsMatrix<T>& b, gsMatrix<T>& x) {
        const index_t n = op_->cols();
        gsMatrix<T> A(op_->rows(), n), e(n, 1), col;
        for (index_t j = 0; j < n; ++j) {
            e.setZero();
            e(j, 0) = T(1);
            op_->apply(e, col);
            for (index_t i = 0; i < A.rows(); ++i) A(i, j) = col(i, 0);
        }
        typename gsSparseSolver<T>::LU lu(A);
        GISMO_ASSERT(lu.info() == gsEigen::Success, "singular block operator");
        x = lu.solve(b);
    }

private:
    OpPtr op_;
};

}  // namespace gismo
