// solvers.h -- device-resident mirrors of gsStaticNewton and the gsALM* arc-length family.
//
// The solver logic (iteration structure, convergence tests, option keys and defaults, the
// Crisfield root selection and complex-root fall-backs) follows the reference classes; the
// vectors live in HBM (FP64, internal order) and the scalars that steer the iteration are
// reduced to the host once per iteration.  The K(u)/R(u) callbacks are the built-in device
// assembler of the problem, and the linear solver is chosen by the "Solver" option.
#pragma once

#include <map>
#include <memory>
#include <string>

#include "linalg.h"
#include "problem.h"

namespace klsa {

struct Options {
    std::map<std::string, double> reals;
    std::map<std::string, int64_t> ints;
    std::map<std::string, std::string> strs;
    double real(const std::string& k, double def) const {
        auto it = reals.find(k);
        if (it != reals.end()) return it->second;
        auto jt = ints.find(k);
        return jt != ints.end() ? (double)jt->second : def;
    }
    int64_t integer(const std::string& k, int64_t def) const {
        auto it = ints.find(k);
        if (it != ints.end()) return it->second;
        auto jt = reals.find(k);
        return jt != reals.end() ? (int64_t)jt->second : def;
    }
    std::string str(const std::string& k, const std::string& def) const {
        auto it = strs.find(k);
        return it != strs.end() ? it->second : def;
    }
};

// gsStaticNewton (gsStaticSolvers/gsStaticNewton.hpp:101-316; options gsStaticBase.h:66-75,
// gsStaticNewton.hpp:20-25).  Residual convention R = L*F - Fint(U).
class StaticNewtonGPU {
public:
    StaticNewtonGPU(Problem& P, const Options& opt);
    int solve_linear();
    int solve();                       // nonlinear Newton
    void set_displacement(const double* d_U);
    void set_update(const double* d_DU);
    void set_load(double L) { L_ = L; }
    const double* solution() const { return U_.get(); }
    int iterations() const { return num_it_; }
    double residual_ratio() const { return residual_ / residualIni_; }
    LinearSolver& lin() { return *S_; }

private:
    void residual(const double* d_x, double* d_R);
    int solve_nonlinear_impl();
    Problem& P_;
    Options opt_;
    std::unique_ptr<LinearSolver> S_;
    DevBuf<double> U_, DU_, dU_, R_, x_, fint_;
    double L_ = 1.0;
    bool headstart_ = false;
    int num_it_ = 0;
    double residual_ = 0, residualIni_ = 1, residualOld_ = 0;
};

// gsALMBase + subclasses (gsALMSolvers/gsALMBase.hpp:22-416, gsALMCrisfield.hpp,
// gsALMRiks.hpp, gsALMLoadControl.hpp, gsALMConsistentCrisfield.hpp).  ALResidual convention
// R = Fint(U) - L*F.
class ALMGPU {
public:
    enum Method { Crisfield = 0, Riks = 1, LoadControl = 2, ConsistentCrisfield = 3 };
    ALMGPU(Problem& P, Method m, const Options& opt);
    void apply_options();
    void initialize(bool stability);
    int step();
    // gsALMBase::computeStability (gsALMBase.hpp:521-545, 547-615) -> gsStatus
    int compute_stability(bool jacobian, double shift);
    double indicator() const { return indicator_; }
    int stability() const { return stability_; }
    bool stability_change() const { return stability_ * stabilityPrev_ < 0; }
    int64_t negatives() const { return negatives_; }
    int bifurcation_method() const { return bifurcation_; }
    // singular points (gsALMBase.hpp:421-512, 628-852); U in internal order on the device
    bool is_bifurcation(bool jacobian);
    int compute_singular_point(const double* d_U, double L, bool switch_branch, bool jacobian, bool test_point);
    void switch_branch();
    const double* V() const { return V_.get(); }
    void set_length(double l);
    double reduce_length(double fac) { arcLength_ *= fac; return arcLength_; }
    double length() const { return arcLength_; }
    void set_solution(const double* d_U, double L);
    void set_solution_step(const double* d_DU, double DL);
    void set_initial_guess(const double* d_U, double L);
    // a guess whose load factor is L + *d_Lcorr, with the correction d_Lcorr still on the device:
    // a placed guess (set_guess_place) reads it with the first residual norms, other uses read
    // it at the start of the step
    void set_initial_guess_dev(const double* d_U, double L, const double* d_Lcorr);
    // gsALMBase::setPrevious (gsALMBase.h:185-191): Uprev, Lprev and DUold = U - Uprev, DLold = L - Lprev
    void set_previous(const double* d_Uprev, double Lprev);
    // distance of a path increment in the method's norm: gsALMCrisfield.h:79-83
    // sqrt(DU.DU + phi^2 F.F DL^2), gsALMRiks.h:81-84 sqrt(phi |DU|^2 + (1 - phi) DL^2); the
    // other methods have none (gsALMBase.h:211-214) and throw
    double distance(const double* d_DU, double DL);
    Method method() const { return method_; }
    const double* U() const { return U_.get(); }
    double L() const { return L_; }
    const double* Uprev() const { return Uprev_.get(); }
    double Lprev() const { return Lprev_; }
    const double* DUold() const { return DUold_.get(); }
    double DLold() const { return DLold_; }
    int iterations() const { return num_it_; }
    double residueF() const { return residueF_; }
    double residueU() const { return residueU_; }
    double phi() const { return phi_; }
    bool converged() const { return converged_; }
    LinearSolver& lin() { return *S_; }
    // Guess placement (no reference counterpart): when set, predictor_guess starts the corrector
    // from the guessed point itself (DU = Uguess - U, DL = Lguess - L) instead of using the guess
    // only for the direction of the tangent predictor (gsALMCrisfield.hpp:167-191).
    void set_guess_place(bool on) { guess_place_ = on; }
    // Frozen tangent after a placed guess (no reference counterpart; option "FrozenIterations",
    // default 0 = off): the first N corrector iterations of a step that starts from a placed guess
    // solve with the factorisation the solver already holds (the last Jacobian of an earlier
    // step, a modified-Newton corrector), then the iteration returns to a fresh Jacobian per
    // iteration.  Used only while the problem's fronts still hold that Jacobian.
    void set_frozen_iterations(int n) { frozen_it_ = n; }
    int max_iter() const { return maxIt_; }
    void set_max_iter(int it) { maxIt_ = it; }
    Problem& problem() { return P_; }
    bool quasi() const { return quasi_; }
    // per-step work counters
    int n_jac = 0, n_res = 0, n_solve = 0;

private:
    void step_impl();
    void initiate_step();
    void predictor();
    void predictor_guess();
    void quasi_newton_iteration();
    void iteration();
    void iteration_finish();
    void compute_jacobian();
    void compute_residual();
    void compute_residual_norms();
    void solve_ut_ubar(bool need_ut);
    void compute_lambda_mu();
    void lambdas_crisfield();
    bool dU_formed_ = false;   // lambdas_crisfield formed dU itself (complex-root branch)
    void consistent_predictor(const double* prevU, double prevL);
    void stability_impl(bool jacobian, double shift);
    bool test_singular_point(bool jacobian);
    void factor64_at(const double* d_x);   // FP64 tangent at x, FP64 fronts
    bool extended_system_solve(double tol);
    void extended_system_iteration();
    bool bisection_solve(double tol);

    Problem& P_;
    Method method_;
    Options opt_;
    std::unique_ptr<LinearSolver> S_;
    int n_;
    DevBuf<double> U_, DU_, dU_, dUt_, dUbar_, DUold_, Uprev_, Uguess_, R_, x_, fint_, rhs2_, sol2_, tmp_;
    DevBuf<double> xjac_;          // point of the last Jacobian (m_jacMat's argument)
    double L_ = 0, DL_ = 0, dL_ = 0, DLold_ = 0, Lprev_ = 0, Lguess_ = 0;
    bool has_guess_ = false;
    const double* Lguess_dev_ = nullptr;   // pending device correction of Lguess_
    const double* Lpending_ = nullptr;     // the correction the current residual still carries
    PinnedBuf<double> Lguess_host_;
    void resolve_guess_load();             // Lguess_ += *Lguess_dev_ (synchronises)
    double FF_ = 0;
    // options
    int maxIt_ = 100;
    double tolF_ = 1e-3, tolU_ = 1e-6, relax_ = 1.0;
    double arcLength_ = 1e-2, arcLength_prev_ = 1e-2, arcLength_ori_ = 1e-2;
    bool adaptive_ = false;
    int desiredIt_ = 10;
    bool quasi_ = false;
    int frozen_it_ = 0;
    uint64_t jac_gen_ = 0;   // generation of the factorisation of the last Jacobian
    int quasiInterval_ = -1;
    double phi_ = -1;
    bool phi_user_ = false;
    int angle_ = 0;
    // state
    int num_it_ = 0;
    bool converged_ = false;
    double eta_ = 1.0;
    double residueF_ = 0, residueU_ = 0, basisF_ = 0, basisU_ = 0;
    bool ut_valid_ = false;
    bool guess_place_ = false;
    // stability (BifurcationMethod -1 nothing, 0 determinant, 1 eigenvalue; gsALMBase.h:385-390)
    int bifurcation_ = 1;
    int stability_ = -1, stabilityPrev_ = -1;
    double indicator_ = 0.0;
    int64_t negatives_ = 0;
    bool fact_stale_ = false;      // the eigenvalue indicator reused the factorisation workspace
    // singular points: options, FP64 solver and extended-system vectors
    double tau_ = 1e3, tolerance_ = 1e-6, spTestTol_ = 1e-6, spTolE_ = 1e-10, spTolB_ = 0.0;
    int spFail_ = 1, spTestIt_ = 5;
    std::unique_ptr<LinearSolver> S64_;
    DevBuf<double> V_, DV_, dV_, ut64_, ub64_, h1_, h2_, Vt_, Vb_, W_, Kv_;
    double residueKTPhi_ = 0.0;
public:
    double residue_ktphi() const { return residueKTPhi_; }
};

}  // namespace klsa
