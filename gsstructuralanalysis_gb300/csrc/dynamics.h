// dynamics.h -- device-resident mirrors of the gsDynamicSolvers time integrators.
//
// The integrators follow gsDynamicSolvers/gsDynamic{Newmark,Bathe,Wilson,ExplicitEuler,
// ImplicitEuler,RK4}.hpp: the same predictor/corrector formulas, Newton loops, convergence tests
// (|dX|/|X| < TolU and |rhs|/|rhs0| < TolF) and option keys with their defaults.  The callbacks
// of the reference (Mass_t, Damping_t, Jacobian_t / Stiffness_t, TResidual_t / TForce_t) are the
// problem's device assembler:
//   M        consistent mass (FP64, on the problem's CSR pattern), assembled once
//   C        Rayleigh damping DampingMass*M + DampingStiffness*K_L (constant; zero by default)
//   K        the tangent K(U) (nonlinear) or the linear stiffness K_L = K(0) (linear)
//   R(U,t)   f(t) F - Fint(U);  Fext(t) = f(t) F, f piecewise linear from a load table
// All vectors are FP64 in the internal (nested-dissection) order and stay on the device; the
// systems M + a C + b K (and M for the explicit integrators) are factorised by the multifrontal
// LDL^T, FP64 fronts by default ("FrontPrecision" 32 selects FP32 fronts with FP64 refinement).
#pragma once

#include <memory>
#include <vector>

#include "linalg.h"
#include "problem.h"
#include "solvers.h"

namespace klsa {

class DynamicGPU {
public:
    enum Method { ExplicitEuler = 0, ImplicitEuler = 1, Newmark = 2, Bathe = 3, Wilson = 4, RK4 = 5 };
    DynamicGPU(Problem& P, Method m, bool nonlinear, const Options& opt);

    // gsDynamicBase::step(dt) (gsDynamicBase.h:196-208): advances the time even when the step fails
    int step(double dt);
    double default_dt() const { return dt_; }
    double time() const { return time_; }
    void set_time(double t) { time_ = t; }
    void set_load_table(const std::vector<double>& t, const std::vector<double>& f);
    double load_factor(double t) const;
    double* U() { return U_.get(); }
    double* V() { return V_.get(); }
    double* A() { return A_.get(); }
    int iterations() const { return iterations_; }

private:
    // integrator bodies on (U, V, A) in place, time t, step dt (the reference's _step_impl)
    int newmark(double t, double dt, double* U, double* V, double* A);
    int bathe(double t, double dt);
    int wilson(double t, double dt);
    int explicit_euler(double t, double dt);
    int implicit_euler(double t, double dt);
    int rk4(double t, double dt);

    // callbacks
    void residual(const double* U, double t, double* R);            // f(t) F - Fint(U)
    void force(double t, double* F);                                 // f(t) F
    void tangent(const double* U);                                   // K_ <- K(U) (or K_L)
    void mass_apply(const double* x, double* y);                     // y = M x
    void damp_apply(const double* x, double* y);                     // y = C x
    void stiff_apply(const double* x, double* y);                    // y = K x
    int factor(double cM, double cC, double cK, bool cacheable);     // cM M + cC C + cK K
    int factor_mass();
    uint64_t generation();                                           // of the problem's fronts
    int solve(const double* b, double* x);
    double norm(const double* x);
    double norm2(const double* x, const double* y);                  // |[x; y]|
    static bool bad(double nrm);                                     // inf or nan
    double* w(int i);                                                // work vector i
    void copy(const double* x, double* y);
    void axpy(double a, const double* x, double* y);                 // y += a x
    void lin(double a, const double* x, double b, const double* y, double* z);   // z = a x + b y

    Problem& P_;
    Method method_;
    bool nl_;
    Options opt_;
    double dt_, tolF_, tolU_, alpha_, delta_, gamma_, cM_, cK_;
    int maxIt_, quasiIt_;
    bool quasi_, fp64_;
    std::unique_ptr<MFSolver> S_;
    DevBuf<double> M_, C_, KL_, K_, lhs_;
    DevBuf<double> U_, V_, A_, fint_;
    DevBuf<double> W_;                   // work vectors, nfree each
    const double* cur_ = nullptr;        // values of the factorised matrix (lhs_ or M_)
    std::vector<double> lt_, lf_;
    double time_ = 0.0;
    int iterations_ = 0;
    // what the factorisation currently holds: 0 nothing, 1 mass, 2 a cacheable combination
    int factored_ = 0;
    double fkey_[3] = {0, 0, 0};
    uint64_t gen_ = 0;
    bool has_damping_ = false;
};

}  // namespace klsa
