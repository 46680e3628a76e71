// linalg.h -- named linear solvers behind the reference's "Solver" option.
#pragma once

#include <memory>
#include <string>

#include "problem.h"

namespace klsa {

// compute()/solve() of gsSparseSolver<T> (gsStaticSolvers/gsStaticNewton.hpp:215-240,
// gsALMSolvers/gsALMBase.hpp:186-211).  Vectors: FP64, internal order, device pointers.
class LinearSolver {
public:
    virtual ~LinearSolver() = default;
    // assemble K at the problem's current displacement and factorise / set up
    virtual int compute_tangent() = 0;
    virtual int solve(const double* d_b, double* d_x, int nrhs) = 0;
    virtual bool has_ldlt() const { return false; }
    virtual void stability(double* min_d, int64_t* neg) { *min_d = 0; *neg = 0; }
    virtual int last_iterations() const { return 0; }
    // x0 = K^-1 (s0 b0), x1 = K^-1 (s1 b1) in one two-right-hand-side solve without staging
    // copies; false when this solver has no such path (the caller stages the pair itself)
    virtual bool solve_pair(const double*, double, const double*, double, double*, double*) { return false; }
    // identifies the factorisation the solver currently holds (0: none / not a factorisation)
    virtual uint64_t generation() const { return 0; }
    // the tangent of the last compute_tangent() sits in the FP64 CSR values (else the FP32 ones)
    virtual bool tangent_values_f64() const { return false; }
};

// Multifrontal LDL^T.  fp64 = false: FP32 fronts (FP32 or FP64-assembled values rounded), with
// optional FP64 iterative refinement against the FP64 values; fp64 = true: FP64 fronts from the
// FP64 values, vectors stay FP64 end to end (option "FrontPrecision" = 64).
class MFSolver : public LinearSolver {
public:
    MFSolver(Problem& P, int refine, double refine_tol, bool fp64 = false);
    int compute_tangent() override;
    int factor_current(bool f64_for_refine);
    int solve(const double* d_b, double* d_x, int nrhs) override;
    bool solve_pair(const double* b0, double s0, const double* b1, double s1, double* x0, double* x1) override;
    bool has_ldlt() const override { return true; }
    void stability(double* min_d, int64_t* neg) override;
    int last_iterations() const override { return last_refine_its_; }
    uint64_t generation() const override;
    bool tangent_values_f64() const override { return tangent_f64_; }
    void set_refine(int r) { refine_ = r; }

private:
    void solve_raw(const double* d_b, double* d_x, int nrhs);
    Problem& P_;
    int refine_;
    double tol_;
    bool fp64_ = false;
    bool has64_ = false;
    bool tangent_f64_ = false;     // precision of the last compute_tangent() assembly
    int last_refine_its_ = 0;
    DevBuf<float> b32_, x32_;
    DevBuf<double> r_, dx_;
};

class PCGSolver : public LinearSolver {
public:
    // block = false: Jacobi (Eigen's DiagonalPreconditioner); true: nodal 3 x 3 block-Jacobi
    PCGSolver(Problem& P, int max_it, double tol, bool block = false);
    int compute_tangent() override;
    int solve(const double* d_b, double* d_x, int nrhs) override;
    int last_iterations() const override { return iterations_; }

private:
    void precondition(const double* r, double* z);
    Problem& P_;
    int max_it_;
    double tol_;
    bool block_;
    int iterations_ = 0, nblk_ = 0;
    DevBuf<double> dinv_, r_, z_, p_, q_, binv_;
    DevBuf<int> blk_start_;
};

std::unique_ptr<LinearSolver> make_linear_solver(Problem& P, const std::string& name, int refine, double refine_tol,
                                                 int cg_max_it, double cg_tol, int front_precision = 32);

}  // namespace klsa
