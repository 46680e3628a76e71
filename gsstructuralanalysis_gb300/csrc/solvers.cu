// solvers.cu -- gsStaticNewton / gsALMCrisfield / gsALMRiks / gsALMLoadControl on the device.
#include "solvers.h"

#include "eigen.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

namespace klsa {

namespace {

struct Fail {
    int code;
};

inline double sgn(double x) { return (double)((x > 0) - (x < 0)); }

std::unique_ptr<LinearSolver> solver_from_options(Problem& P, const Options& opt, const std::string& def) {
    std::string name = opt.str("Solver", def);
    auto s = make_linear_solver(P, name, (int)opt.integer("Refinement", 0), opt.real("RefineTol", 1e-12),
                                (int)opt.integer("CGMaxIterations", 0), opt.real("CGTolerance", 1e-10),
                                (int)opt.integer("FrontPrecision", 32));
    if (!s) throw std::invalid_argument("unknown Solver '" + name + "'");
    return s;
}

}  // namespace

// ------------------------------------------------------------------------------------------
// gsStaticNewton
// ------------------------------------------------------------------------------------------
StaticNewtonGPU::StaticNewtonGPU(Problem& P, const Options& opt) : P_(P), opt_(opt) {
    // gsStaticNewton::defaultOptions sets Solver = CGDiagonal (gsStaticNewton.hpp:23)
    S_ = solver_from_options(P_, opt_, "CGDiagonal");
    int n = P_.nfree;
    U_.alloc(n); DU_.alloc(n); dU_.alloc(n); R_.alloc(n); x_.alloc(n); fint_.alloc(n);
    U_.zero(P_.stream); DU_.zero(P_.stream); dU_.zero(P_.stream);
}

void StaticNewtonGPU::residual(const double* d_x, double* d_R) {
    P_.set_displacement(d_x);
    P_.internal_force(fint_.get());
    vec::lincomb(L_, P_.d_F.get(), -1.0, fint_.get(), d_R, P_.nfree, P_.stream);
}

int StaticNewtonGPU::solve_linear() {
    KL_CUDA(cudaMemsetAsync(x_.get(), 0, sizeof(double) * P_.nfree, P_.stream));
    P_.set_displacement(x_.get());
    int st = S_->compute_tangent();
    if (st != ST_SUCCESS) return ST_SOLVER_ERROR;
    vec::lincomb(L_, P_.d_F.get(), 0.0, P_.d_F.get(), R_.get(), P_.nfree, P_.stream);
    return S_->solve(R_.get(), U_.get(), 1) == ST_SUCCESS ? ST_SUCCESS : ST_SOLVER_ERROR;
}

void StaticNewtonGPU::set_displacement(const double* d_U) {
    KL_CUDA(cudaMemcpyAsync(U_.get(), d_U, sizeof(double) * P_.nfree, cudaMemcpyDeviceToDevice, P_.stream));
}

void StaticNewtonGPU::set_update(const double* d_DU) {
    KL_CUDA(cudaMemcpyAsync(DU_.get(), d_DU, sizeof(double) * P_.nfree, cudaMemcpyDeviceToDevice, P_.stream));
    headstart_ = true;
}

int StaticNewtonGPU::solve_nonlinear_impl() {
    const int n = P_.nfree;
    cudaStream_t s = P_.stream;
    double tol = opt_.real("tol", 1e-6);
    double tolF = opt_.real("tolF", -1) != -1 ? opt_.real("tolF", -1) : tol;
    double tolU = opt_.real("tolU", -1) != -1 ? opt_.real("tolU", -1) : tol;
    int maxIt = (int)opt_.integer("maxIt", 25);
    double relax = opt_.real("Relaxation", 1.0);
    // gsStaticNewton.hpp:148-153 takes a linear head start only while m_DeltaU has no rows.  The
    // reference's drivers construct the solver and call initialize() (gsStaticBase.h:53-57), whose
    // reset() sizes m_DeltaU to the dofs (gsStaticBase.h:136-144), so that branch never runs: the
    // iteration starts from U with a zero increment.  This solver is created in that state.
    // _start (hpp:274-316)
    if (!headstart_) {
        KL_CUDA(cudaMemsetAsync(DU_.get(), 0, sizeof(double) * n, s));
        residual(U_.get(), R_.get());
        double rr;
        const double* a[1] = {R_.get()};
        vec::multidot(1, a, a, n, &rr, s);
        residual_ = std::sqrt(rr);
        if (residual_ == 0) residual_ = 1;
        residualIni_ = residualOld_ = residual_;
    } else {
        vec::lincomb(1.0, U_.get(), 1.0, DU_.get(), x_.get(), n, s);
        residual(x_.get(), R_.get());
        double rr;
        const double* a[1] = {R_.get()};
        vec::multidot(1, a, a, n, &rr, s);
        residual_ = std::sqrt(rr);
        if (residual_ == 0) residual_ = 1;
        residualOld_ = residual_;
        DevBuf<double> R0(n);
        residual(U_.get(), R0.get());
        const double* b[1] = {R0.get()};
        vec::multidot(1, b, b, n, &rr, s);
        residualIni_ = std::sqrt(rr);
        if (residualIni_ == 0) residualIni_ = 1;
        headstart_ = false;
    }
    KL_CUDA(cudaMemsetAsync(dU_.get(), 0, sizeof(double) * n, s));
    for (num_it_ = 0; num_it_ != maxIt; ++num_it_) {
        vec::lincomb(1.0, U_.get(), 1.0, DU_.get(), x_.get(), n, s);
        P_.set_displacement(x_.get());
        if (S_->compute_tangent() != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        if (S_->solve(R_.get(), dU_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        vec::axpby(relax, dU_.get(), 1.0, DU_.get(), n, s);
        vec::lincomb(1.0, U_.get(), 1.0, DU_.get(), x_.get(), n, s);
        residual(x_.get(), R_.get());
        double d[3];
        const double* xs[3] = {R_.get(), dU_.get(), DU_.get()};
        vec::multidot(3, xs, xs, n, d, s);
        residual_ = std::sqrt(d[0]);
        residualOld_ = residual_;
        double ratioU = relax * std::sqrt(d[1]) / std::sqrt(d[2]);
        if (ratioU < tolU && residual_ / residualIni_ < tolF) {
            vec::axpby(1.0, DU_.get(), 1.0, U_.get(), n, s);
            break;
        } else if (num_it_ + 1 == maxIt) {
            vec::axpby(1.0, DU_.get(), 1.0, U_.get(), n, s);
            throw Fail{ST_NOT_CONVERGED};
        }
    }
    return ST_SUCCESS;
}

int StaticNewtonGPU::solve() {
    try {
        return solve_nonlinear_impl();
    } catch (const Fail& f) {
        return f.code;
    }
}

// ------------------------------------------------------------------------------------------
// arc-length family
// ------------------------------------------------------------------------------------------
ALMGPU::ALMGPU(Problem& P, Method m, const Options& opt) : P_(P), method_(m), opt_(opt) {
    // gsALMBase::defaultOptions: Solver = SimplicialLDLT (gsALMBase.hpp:48)
    S_ = solver_from_options(P_, opt_, "SimplicialLDLT");
    n_ = P_.nfree;
    for (DevBuf<double>* b : {&U_, &DU_, &dU_, &dUt_, &dUbar_, &DUold_, &Uprev_, &Uguess_, &R_, &x_, &fint_, &tmp_, &xjac_}) {
        b->alloc(n_);
        b->zero(P_.stream);
    }
    rhs2_.alloc(2 * (size_t)n_);
    sol2_.alloc(2 * (size_t)n_);
    apply_options();
    const double* f[1] = {P_.d_F.get()};
    vec::multidot(1, f, f, n_, &FF_, P_.stream);
}

void ALMGPU::apply_options() {
    maxIt_ = (int)opt_.integer("MaxIter", 100);
    tolF_ = opt_.real("TolF", 1e-3);
    tolU_ = opt_.real("TolU", 1e-6);
    arcLength_ = arcLength_prev_ = arcLength_ori_ = opt_.real("Length", 1e-2);
    adaptive_ = opt_.integer("AdaptiveLength", 0) != 0;
    desiredIt_ = (int)opt_.integer("AdaptiveIterations", 10);
    quasi_ = opt_.integer("Quasi", 0) != 0;
    quasiInterval_ = (int)opt_.integer("QuasiIterations", -1);
    frozen_it_ = (int)opt_.integer("FrozenIterations", 0);
    relax_ = opt_.real("Relaxation", 1.0);
    phi_ = opt_.real("Scaling", -1.0);
    phi_user_ = phi_ != -1.0;
    angle_ = (int)opt_.integer("AngleMethod", 0);
    // gsALMBase.hpp:39, 72-78: Eigenvalue by default; Determinant needs the LDL^T solver
    bifurcation_ = (int)opt_.integer("BifurcationMethod", 1);
    if (bifurcation_ == 0 && !S_->has_ldlt()) bifurcation_ = 1;
    // singular-point options (gsALMBase.hpp:26-45, 60-90)
    tolerance_ = opt_.real("Tol", 1e-6);
    tau_ = opt_.real("Perturbation", 1e3);
    spFail_ = (int)opt_.integer("SingularPointFailure", 1);
    spTestTol_ = opt_.real("SingularPointTestTol", 1e-6);
    spTestIt_ = (int)opt_.integer("SingularPointTestIt", 5);
    spTolE_ = opt_.real("SingularPointComputeTolE", 1e-10);
    spTolB_ = opt_.real("SingularPointComputeTolB", 0.0);
}

void ALMGPU::set_length(double l) {
    opt_.reals["Length"] = l;
    arcLength_ = arcLength_prev_ = arcLength_ori_ = l;
}

void ALMGPU::initialize(bool stability) {
    for (DevBuf<double>* b : {&U_, &DU_, &DUold_, &Uprev_}) b->zero(P_.stream);
    L_ = DL_ = DLold_ = Lprev_ = 0.0;
    // gsALMBase::init (gsALMBase.hpp:95-103): stability at U with a fresh Jacobian
    if (stability) stability_impl(true, -1e2);
}

void ALMGPU::stability_impl(bool jacobian, double shift) {
    if (jacobian) {
        // Jacobian at U, factorised (gsALMBase.hpp:549-554)
        KL_CUDA(cudaMemcpyAsync(xjac_.get(), U_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, P_.stream));
        P_.set_displacement(xjac_.get());
        ++n_jac;
        if (S_->compute_tangent() != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        ut_valid_ = false;
        fact_stale_ = false;
        jac_gen_ = S_->generation();
    }
    if (bifurcation_ == 0) {
        // Determinant (gsALMBase.hpp:557-569): D of the current LDL^T factorisation
        double mn = 0.0;
        int64_t neg = 0;
        S_->stability(&mn, &neg);
        indicator_ = mn;
        negatives_ = neg;
    } else if (bifurcation_ == 1) {
        // Eigenvalue (gsALMBase.hpp:570-598): nev = min(floor(n/5), 10), ncv = 5 nev, tol 1e-6, on
        // the Jacobian of the last iteration, evaluated in FP64
        int number = std::min(n_ / 5, 10);
        if (number < 1) throw Fail{ST_SOLVER_ERROR};
        P_.set_displacement(xjac_.get());
        P_.tangent_f64();
        std::vector<double> vals(number);
        int st = standard_eigs_gpu(P_, P_.d_vals64.get(), number, 5, shift, 1e-6, vals.data());
        fact_stale_ = true;
        if (st != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        negatives_ = std::count_if(vals.begin(), vals.end(), [](double v) { return v < 0; });
        indicator_ = *std::min_element(vals.begin(), vals.end());
    } else {
        indicator_ = 0.0;
        negatives_ = 0;
    }
    stability_ = indicator_ < 0 ? 1 : -1;
}

int ALMGPU::compute_stability(bool jacobian, double shift) {
    try {
        stability_impl(jacobian, shift);
        return ST_SUCCESS;
    } catch (const Fail& f) {
        return f.code;
    }
}

void ALMGPU::set_solution(const double* d_U, double L) {
    KL_CUDA(cudaMemcpyAsync(U_.get(), d_U, sizeof(double) * n_, cudaMemcpyDeviceToDevice, P_.stream));
    L_ = L;
}

void ALMGPU::set_solution_step(const double* d_DU, double DL) {
    KL_CUDA(cudaMemcpyAsync(DUold_.get(), d_DU, sizeof(double) * n_, cudaMemcpyDeviceToDevice, P_.stream));
    DLold_ = DL;
}

void ALMGPU::set_previous(const double* d_Uprev, double Lprev) {
    KL_CUDA(cudaMemcpyAsync(Uprev_.get(), d_Uprev, sizeof(double) * n_, cudaMemcpyDeviceToDevice, P_.stream));
    Lprev_ = Lprev;
    vec::lincomb(1.0, U_.get(), -1.0, Uprev_.get(), DUold_.get(), n_, P_.stream);
    DLold_ = L_ - Lprev_;
}

double ALMGPU::distance(const double* d_DU, double DL) {
    double uu = 0.0;
    vec::multidot(1, &d_DU, &d_DU, n_, &uu, P_.stream);
    if (method_ == Crisfield) return std::sqrt(uu + phi_ * phi_ * FF_ * DL * DL);
    if (method_ == Riks) return std::sqrt(phi_ * uu + (1.0 - phi_) * DL * DL);
    throw std::invalid_argument("distance: not defined for this arc-length method");
}

void ALMGPU::set_initial_guess(const double* d_U, double L) {
    KL_CUDA(cudaMemcpyAsync(Uguess_.get(), d_U, sizeof(double) * n_, cudaMemcpyDeviceToDevice, P_.stream));
    Lguess_ = L;
    Lguess_dev_ = nullptr;
    has_guess_ = true;
}

void ALMGPU::set_initial_guess_dev(const double* d_U, double L, const double* d_Lcorr) {
    set_initial_guess(d_U, L);
    Lguess_dev_ = d_Lcorr;
}

void ALMGPU::resolve_guess_load() {
    if (!Lguess_dev_) return;
    KL_CUDA(cudaMemcpyAsync(Lguess_host_.get(), Lguess_dev_, sizeof(double), cudaMemcpyDeviceToHost, P_.stream));
    KL_CUDA(cudaStreamSynchronize(P_.stream));
    Lguess_ += *Lguess_host_.get();
    Lguess_dev_ = nullptr;
}

void ALMGPU::compute_jacobian() {
    P_.set_displacement_sum(U_.get(), DU_.get(), x_.get());
    ++n_jac;
    if (S_->compute_tangent() != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
    KL_CUDA(cudaMemcpyAsync(xjac_.get(), x_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, P_.stream));
    ut_valid_ = false;
    fact_stale_ = false;
    jac_gen_ = S_->generation();
}

void ALMGPU::compute_residual() {
    cudaEvent_t ev = g_timer.begin(P_.stream);
    P_.set_displacement_sum(U_.get(), DU_.get(), x_.get());
    // ALResidual: Fint - (L + DL) F; a placed guess may still carry its load correction on the device
    P_.internal_force(R_.get(), -(L_ + DL_), P_.d_F.get(), Lpending_);
    g_timer.end(P_.stream, 3, ev);
    ++n_res;
}

void ALMGPU::compute_residual_norms() {
    double d[3];
    const double* xs[3] = {R_.get(), dU_.get(), DU_.get()};
    if (Lpending_)   // read with the norms (the reduction synchronises the stream)
        KL_CUDA(cudaMemcpyAsync(Lguess_host_.get(), Lpending_, sizeof(double), cudaMemcpyDeviceToHost, P_.stream));
    vec::multidot(3, xs, xs, n_, d, P_.stream);
    if (Lpending_) {
        const double c = *Lguess_host_.get();
        Lguess_ += c;
        DL_ += c;
        dL_ += c;
        Lpending_ = nullptr;
    }
    double nR = std::sqrt(d[0]), ndU = std::sqrt(d[1]), nDU = std::sqrt(d[2]);
    if (num_it_ == 0) {
        basisF_ = std::fabs(L_ + DL_) * std::sqrt(FF_);
        basisU_ = nDU;
        residueF_ = nR / basisF_;
        residueU_ = ndU / nDU;
    } else {
        residueF_ = nR / basisF_;
        residueU_ = ndU / basisU_;
    }
}

// one factorisation, two right-hand sides: [F, -R] -> [dUt, dUbar]
void ALMGPU::solve_ut_ubar(bool need_ut) {
    cudaStream_t s = P_.stream;
    if (need_ut && S_->solve_pair(P_.d_F.get(), 1.0, R_.get(), -1.0, dUt_.get(), dUbar_.get())) {
        n_solve += 2;
        ut_valid_ = true;
    } else if (need_ut) {
        KL_CUDA(cudaMemcpyAsync(rhs2_.get(), P_.d_F.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        vec::lincomb(-1.0, R_.get(), 0.0, R_.get(), rhs2_.get() + n_, n_, s);
        if (S_->solve(rhs2_.get(), sol2_.get(), 2) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        KL_CUDA(cudaMemcpyAsync(dUt_.get(), sol2_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        KL_CUDA(cudaMemcpyAsync(dUbar_.get(), sol2_.get() + n_, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        n_solve += 2;
        ut_valid_ = true;
    } else {
        vec::lincomb(-1.0, R_.get(), 0.0, R_.get(), rhs2_.get(), n_, s);
        if (S_->solve(rhs2_.get(), dUbar_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        n_solve += 1;
    }
}

void ALMGPU::initiate_step() {
    const bool cr = method_ == Crisfield;
    vec::zero4(DU_.get(), dU_.get(), cr ? dUbar_.get() : nullptr, cr ? dUt_.get() : nullptr, n_, P_.stream);
    if (cr) eta_ = 1.0;
    DL_ = dL_ = 0.0;
}

void ALMGPU::compute_lambda_mu() {
    // gsALMCrisfield.hpp:384-398
    double A0 = phi_ * phi_ * FF_;
    double d[2];
    const double* xs[2] = {DUold_.get(), dUt_.get()};
    const double* ys[2] = {dUt_.get(), dUt_.get()};
    vec::multidot(2, xs, ys, n_, d, P_.stream);
    double dir = sgn(d[0] + A0 * DLold_);
    double denum = std::sqrt(d[1] + A0);
    double mu = denum == 0 ? arcLength_ : arcLength_ / denum;
    dL_ = dir * mu;
    vec::lincomb(dL_, dUt_.get(), 0.0, dUt_.get(), dU_.get(), n_, P_.stream);
}

void ALMGPU::predictor() {
    cudaStream_t s = P_.stream;
    compute_jacobian();
    if (method_ == Crisfield) {
        if (S_->solve(P_.d_F.get(), dUt_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        ++n_solve;
        ut_valid_ = true;
        double d[3];
        const double* xs[3] = {DUold_.get(), dUt_.get(), U_.get()};
        vec::multidot(3, xs, xs, n_, d, s);
        if (d[0] == 0 && DLold_ * DLold_ == 0) {
            dL_ = arcLength_ / std::sqrt(2 * d[1]);
            vec::lincomb(1.0, dUbar_.get(), dL_, dUt_.get(), dU_.get(), n_, s);
            if (!phi_user_) phi_ = std::sqrt(d[1] / FF_);
        } else {
            if (!phi_user_) phi_ = std::sqrt(d[2] / (L_ * L_ * FF_));
            compute_lambda_mu();
        }
        vec::axpby(1.0, dU_.get(), 1.0, DU_.get(), n_, s);
        DL_ += dL_;
        if (angle_ == 1 || angle_ == 2) {
            KL_CUDA(cudaMemcpyAsync(DUold_.get(), DU_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
            DLold_ = DL_;
        }
    } else if (method_ == Riks) {
        phi_ = n_ == 1 ? 0.99999999999 : 1.0 / n_;
        double d[1];
        vec::lincomb(1.0, U_.get(), -1.0, Uprev_.get(), tmp_.get(), n_, s);
        const double* xs[1] = {tmp_.get()};
        vec::multidot(1, xs, xs, n_, d, s);
        const double tol = 1e-10;
        if (std::sqrt(d[0]) < tol && (L_ - Lprev_) * (L_ - Lprev_) < tol) {
            double DLs = 1.0;
            if (S_->solve(P_.d_F.get(), dUt_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
            ++n_solve;
            ut_valid_ = true;
            double uu;
            const double* a[1] = {dUt_.get()};
            vec::multidot(1, a, a, n_, &uu, s);
            double den = std::sqrt(uu + DL_ * DLs);
            vec::lincomb(1.0 / den, dUt_.get(), 0.0, dUt_.get(), dU_.get(), n_, s);
            dL_ = DLs / den;
        } else {
            dL_ = (L_ - Lprev_) / arcLength_prev_;
            vec::lincomb(1.0 / arcLength_prev_, tmp_.get(), 0.0, tmp_.get(), dU_.get(), n_, s);
        }
        dL_ *= arcLength_;
        vec::axpby(0.0, dU_.get(), arcLength_, dU_.get(), n_, s);
        vec::axpby(1.0, dU_.get(), 1.0, DU_.get(), n_, s);
        DL_ += dL_;
    } else if (method_ == ConsistentCrisfield) {
        // gsALMConsistentCrisfield.hpp:104-146: tangent direction on the first step, secant
        // (U - Uprev, L - Lprev) / l_prev afterwards; phi from the last u_t
        consistent_predictor(Uprev_.get(), Lprev_);
    } else {  // LoadControl
        DL_ = dL_ = arcLength_;
        if (S_->solve(P_.d_F.get(), dUt_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        ++n_solve;
        vec::lincomb(dL_, dUt_.get(), 0.0, dUt_.get(), DU_.get(), n_, s);
    }
}

void ALMGPU::predictor_guess() {
    cudaStream_t s = P_.stream;
    if (guess_place_) {
        // start the corrector at the guess: no tangent at U, no u_t solve
        vec::lincomb_ext(1.0, Uguess_.get(), -1.0, U_.get(), DU_.get(), dU_.get(), nullptr, n_, s);
        DL_ = dL_ = Lguess_ - L_;
        ut_valid_ = false;
        has_guess_ = false;
        return;
    }
    compute_jacobian();
    if (method_ == Crisfield) {
        // gsALMCrisfield.hpp:167-191
        if (S_->solve(P_.d_F.get(), dUt_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        ++n_solve;
        ut_valid_ = true;
        double uu;
        const double* a[1] = {dUt_.get()};
        vec::multidot(1, a, a, n_, &uu, s);
        if (!phi_user_) phi_ = std::sqrt(uu / FF_);
        vec::lincomb(-1.0, Uguess_.get(), 1.0, U_.get(), DUold_.get(), n_, s);
        DLold_ = -(Lguess_ - L_);
        compute_lambda_mu();
        KL_CUDA(cudaMemcpyAsync(DU_.get(), dU_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        DL_ = dL_;
    } else if (method_ == Riks) {
        if (S_->solve(P_.d_F.get(), dUt_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        ++n_solve;
        ut_valid_ = true;
        vec::lincomb(1.0, Uguess_.get(), -1.0, U_.get(), tmp_.get(), n_, s);
        double d;
        const double* a[1] = {tmp_.get()};
        vec::multidot(1, a, a, n_, &d, s);
        const double tol = 1e-10;
        if (std::sqrt(d) < tol && (Lguess_ - L_) * (Lguess_ - L_) < tol) {
            double uu;
            const double* b[1] = {dUt_.get()};
            vec::multidot(1, b, b, n_, &uu, s);
            double den = std::sqrt(uu + DL_);
            vec::lincomb(1.0 / den, dUt_.get(), 0.0, dUt_.get(), dU_.get(), n_, s);
            dL_ = 1.0 / den;
        } else {
            dL_ = (Lguess_ - L_) / arcLength_prev_;
            vec::lincomb(1.0 / arcLength_prev_, tmp_.get(), 0.0, tmp_.get(), dU_.get(), n_, s);
        }
        dL_ *= arcLength_;
        vec::axpby(0.0, dU_.get(), arcLength_, dU_.get(), n_, s);
        KL_CUDA(cudaMemcpyAsync(DU_.get(), dU_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        DL_ = dL_;
    } else if (method_ == ConsistentCrisfield) {
        // gsALMConsistentCrisfield.hpp:148-190: the same with (Uguess - U, Lguess - L)
        consistent_predictor(nullptr, 0.0);
    } else {
        DL_ = dL_ = Lguess_ - L_;
        if (S_->solve(P_.d_F.get(), dUt_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        ++n_solve;
        vec::lincomb(dL_, dUt_.get(), 0.0, dUt_.get(), DU_.get(), n_, s);
    }
    has_guess_ = false;
}

// Predictor of gsALMConsistentCrisfield (Jacobian already factorised).  With `prevU` the secant
// is (U - prevU, L - prevL) (predictor); with null it is (Uguess - U, Lguess - L) (predictorGuess).
void ALMGPU::consistent_predictor(const double* prevU, double prevL) {
    cudaStream_t s = P_.stream;
    if (prevU) {
        vec::lincomb(1.0, U_.get(), -1.0, prevU, tmp_.get(), n_, s);
    } else {
        vec::lincomb(1.0, Uguess_.get(), -1.0, U_.get(), tmp_.get(), n_, s);
    }
    const double dLsec = prevU ? (L_ - prevL) : (Lguess_ - L_);
    double d[2];
    const double* xs[2] = {tmp_.get(), dUt_.get()};
    vec::multidot(2, xs, xs, n_, d, s);
    const double tol = 1e-10;
    if (std::sqrt(d[0]) < tol && dLsec * dLsec < tol) {
        const double DLs = 1.0;
        if (S_->solve(P_.d_F.get(), dUt_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        ++n_solve;
        ut_valid_ = true;
        double uu;
        const double* a[1] = {dUt_.get()};
        vec::multidot(1, a, a, n_, &uu, s);
        const double den = std::sqrt(uu + DL_ * DLs);
        vec::lincomb(1.0 / den, dUt_.get(), 0.0, dUt_.get(), dU_.get(), n_, s);
        dL_ = DLs / den;
        if (!phi_user_) phi_ = std::sqrt(uu / FF_);
    } else {
        dL_ = dLsec / arcLength_prev_;
        vec::lincomb(1.0 / arcLength_prev_, tmp_.get(), 0.0, tmp_.get(), dU_.get(), n_, s);
        if (!phi_user_) phi_ = std::sqrt(d[1] / FF_);
    }
    dL_ *= arcLength_;
    vec::axpby(0.0, dU_.get(), arcLength_, dU_.get(), n_, s);
    vec::axpby(1.0, dU_.get(), 1.0, DU_.get(), n_, s);
    DL_ += dL_;
}

void ALMGPU::quasi_newton_iteration() {
    compute_jacobian();
}

void ALMGPU::lambdas_crisfield() {
    // gsALMCrisfield.hpp:213-427 (computeLambdas, Simple, Modified, Eta, Complex, DOT)
    cudaStream_t s = P_.stream;
    double A0 = phi_ * phi_ * FF_;
    double d[7];
    const double* xs[7] = {dUt_.get(), dUt_.get(), dUbar_.get(), DU_.get(), DU_.get(), dUbar_.get(), DUold_.get()};
    const double* ys[7] = {dUt_.get(), DU_.get(), dUt_.get(), DU_.get(), dUbar_.get(), dUbar_.get(), dUt_.get()};
    vec::multidot(7, xs, ys, n_, d, s);
    double a0 = d[0] + A0;
    double b0 = 2 * (d[1] + DL_ * A0);
    double b1 = 2 * d[2];
    double c0 = d[3] + DL_ * DL_ * A0 - arcLength_ * arcLength_;
    double c1 = 2 * d[4];
    double c2 = d[5];
    double DOTfac = d[6] + phi_ * phi_ * DLold_;
    double al1 = a0, al2 = b0 + eta_ * b1, al3 = c0 + eta_ * c1 + eta_ * eta_ * c2;
    double disc = al2 * al2 - 4 * al1 * al3;
    // the root's update dU = eta dUbar + dL dUt is formed by the caller (with DU += dU in the
    // same pass); only the complex-root branch below forms dU itself (dU_formed_)
    dU_formed_ = false;
    auto choose = [&](double r0, double r1) {
        double d0 = r0 * DOTfac, d1 = r1 * DOTfac;
        double r = (d0 < d1) ? r1 : r0;
        dL_ = r;
    };
    if (disc >= 0) {
        eta_ = 1.0;
        choose((-al2 + std::sqrt(disc)) / (2 * al1), (-al2 - std::sqrt(disc)) / (2 * al1));
        return;
    }
    // modified (Lam 1992)
    al1 = b1 * b1 - 4.0 * a0 * c2;
    al2 = 2.0 * b0 * b1 - 4.0 * a0 * c1;
    al3 = b0 * b0 - 4.0 * a0 * c0;
    disc = al2 * al2 - 4.0 * al1 * al3;
    if (disc >= 0) {
        double e0 = (-al2 + std::sqrt(disc)) / (2.0 * al1), e1 = (-al2 - std::sqrt(disc)) / (2.0 * al1);
        double eta1 = std::min(e0, e1), eta2 = std::max(e0, e1);
        double xi = 0.05 * std::fabs(eta2 - eta1);
        if (eta2 < 1.0) eta_ = eta2 - xi;
        else if (eta2 > 1.0 && -al2 / al1 < 1.0) eta_ = eta2 + xi;
        else if (eta1 < 1.0 && -al2 / al1 > 1.0) eta_ = eta1 - xi;
        else if (eta1 > 1.0) eta_ = eta1 + xi;
    }
    if (disc >= 0 && eta_ > 0.05) {
        double bl1 = a0, bl2 = b0 + eta_ * b1;
        double r = -bl2 / (2 * bl1);
        choose(r, r);
        return;
    }
    // simplified complex-root solve (Lam 1992 eq. 13-17)
    eta_ = 1.0;
    vec::lincomb(1.0, U_.get(), 1.0, DU_.get(), x_.get(), n_, s);
    spmv(P_, S_->tangent_values_f64(), x_.get(), tmp_.get());   // Fint ~ K (U + DU), the current tangent
    double fF;
    const double* fa[1] = {tmp_.get()};
    const double* fb[1] = {P_.d_F.get()};
    vec::multidot(1, fa, fb, n_, &fF, s);
    double Lcr = fF / FF_;
    double DLcr = Lcr - L_;
    double DUcr2 = d[3] + 2 * d[4] + d[5];              // (DU + dUbar).(DU + dUbar)
    double arc_cr = std::sqrt(DUcr2 + A0 * DLcr * DLcr);
    double mu = arcLength_ / arc_cr;
    dL_ = mu * DLcr - DL_;
    // dU = mu (DU + dUbar) - DU
    vec::lincomb(mu - 1.0, DU_.get(), mu, dUbar_.get(), dU_.get(), n_, s);
    dU_formed_ = true;
}

void ALMGPU::iteration() {
    cudaStream_t s = P_.stream;
    if (fact_stale_) {
        // a quasi-Newton iteration after an eigenvalue stability test: refactorise the Jacobian
        P_.set_displacement(xjac_.get());
        ++n_jac;
        if (S_->compute_tangent() != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        fact_stale_ = false;
        jac_gen_ = S_->generation();
    }
    if (method_ == Crisfield) {
        solve_ut_ubar(!ut_valid_);
        eta_ = 1.0;
        double lamold = dL_;
        lambdas_crisfield();
        if ((lamold * dL_ < 0 && std::fabs(dL_) <= std::fabs(lamold)) && relax_ != 1.0) {
            vec::lincomb_ext(relax_ * dL_, dUt_.get(), relax_ * eta_, dUbar_.get(), dU_.get(), nullptr, DU_.get(), n_, s);
            dL_ = relax_ * dL_;
        } else if (!dU_formed_) {
            vec::lincomb_ext(eta_, dUbar_.get(), dL_, dUt_.get(), dU_.get(), nullptr, DU_.get(), n_, s);
        } else {
            vec::axpby(1.0, dU_.get(), 1.0, DU_.get(), n_, s);
        }
        DL_ += dL_;
        if (angle_ == 1) {
            KL_CUDA(cudaMemcpyAsync(DUold_.get(), DU_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
            DLold_ = DL_;
        }
    } else if (method_ == ConsistentCrisfield) {
        // gsALMConsistentCrisfield.hpp:75-90 (Carrera 1994, eqs. 20-21)
        solve_ut_ubar(!ut_valid_);
        double d[3];
        const double* xs[3] = {DU_.get(), DU_.get(), DU_.get()};
        const double* ys[3] = {DU_.get(), dUbar_.get(), dUt_.get()};
        vec::multidot(3, xs, ys, n_, d, s);
        const double cres = d[0] + phi_ * phi_ * DL_ * DL_ * FF_ - arcLength_ * arcLength_;
        const double num = cres + 2.0 * d[1];
        const double denum = 2.0 * d[2] + phi_ * phi_ * 2.0 * DL_ * FF_;
        dL_ = -num / denum;
        vec::lincomb(dL_, dUt_.get(), 1.0, dUbar_.get(), dU_.get(), n_, s);
        vec::axpby(1.0, dU_.get(), 1.0, DU_.get(), n_, s);
        DL_ += dL_;
    } else if (method_ == Riks) {
        solve_ut_ubar(!ut_valid_);
        double d[3];
        const double* xs[3] = {DU_.get(), DU_.get(), DU_.get()};
        const double* ys[3] = {DU_.get(), dUbar_.get(), dUt_.get()};
        vec::multidot(3, xs, ys, n_, d, s);
        double r = phi_ * d[0] + (1 - phi_) * DL_ * DL_ - arcLength_ * arcLength_;
        dL_ = -(r + 2 * phi_ * d[1]) / (2 * (1 - phi_) * DL_ + 2 * phi_ * d[2]);
        vec::lincomb(1.0, dUbar_.get(), dL_, dUt_.get(), dU_.get(), n_, s);
        vec::axpby(1.0, dU_.get(), 1.0, DU_.get(), n_, s);
        DL_ += dL_;
    } else {
        solve_ut_ubar(false);
        KL_CUDA(cudaMemcpyAsync(dU_.get(), dUbar_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        vec::axpby(1.0, dU_.get(), 1.0, DU_.get(), n_, s);
    }
}

void ALMGPU::iteration_finish() {
    cudaStream_t s = P_.stream;
    converged_ = true;
    const bool keep_old = (method_ == Crisfield && angle_ == 0) || method_ == ConsistentCrisfield;
    vec::step_finish(U_.get(), DU_.get(), Uprev_.get(), keep_old ? DUold_.get() : nullptr, n_, s);   // Uprev = U; U += DU
    Lprev_ = L_;
    L_ += DL_;
    if (keep_old) DLold_ = DL_;
}

void ALMGPU::step_impl() {
    converged_ = false;
    num_it_ = 0;
    initiate_step();
    // gsALMBase.hpp:365: the guess is used when (Uguess - U).norm() != 0 and Lguess != L.  A placed
    // guess starts the corrector at DU = Uguess - U, whose norm comes back with the residual norms:
    // the test is made there, and the step restarts from the tangent predictor if it fails.
    bool use_guess = false, check_placed = false;
    Lpending_ = nullptr;
    if (has_guess_ && !guess_place_) resolve_guess_load();
    if (has_guess_ && (Lguess_dev_ || (Lguess_ - L_) != 0)) {
        if (guess_place_) {
            use_guess = check_placed = true;
            Lpending_ = Lguess_dev_;   // DL below lacks this correction until the first residual norms
            Lguess_dev_ = nullptr;
        } else {
            double d;
            vec::lincomb(1.0, Uguess_.get(), -1.0, U_.get(), tmp_.get(), n_, P_.stream);
            const double* a[1] = {tmp_.get()};
            vec::multidot(1, a, a, n_, &d, P_.stream);
            use_guess = d != 0;
        }
    }
    // frozen tangent: a placed guess, and the fronts still hold this solver's last Jacobian
    bool frozen = use_guess && guess_place_ && frozen_it_ > 0 && S_->has_ldlt() && !fact_stale_ &&
                  jac_gen_ != 0 && jac_gen_ == S_->generation();
    if (use_guess) predictor_guess();
    else predictor();
    compute_residual();
    compute_residual_norms();
    if (check_placed && (basisU_ == 0 || DL_ == 0)) {   // Uguess == U or Lguess == L
        frozen = false;
        initiate_step();
        predictor();
        compute_residual();
        compute_residual_norms();
    }
    if (quasi_) {
        // quasiNewtonPredictor (gsALMCrisfield.hpp:56-63, gsALMRiks.hpp:38-45,
        // gsALMLoadControl.hpp:23-29): the Jacobian at the predicted point U + DU, kept for the
        // iterations; u_t and u_bar follow from it in iteration()
        compute_jacobian();
    }
    stabilityPrev_ = stability_;
    for (num_it_ = 1; num_it_ < maxIt_; ++num_it_) {
        bool refresh = !quasi_ || (quasiInterval_ > 0 && num_it_ % quasiInterval_ == 0);
        if (frozen && num_it_ <= frozen_it_) refresh = false;
        if (refresh) quasi_newton_iteration();
        iteration();
        stability_impl(false, -1e2);   // gsALMBase.hpp:390
        compute_residual();
        compute_residual_norms();
        if (residueF_ < tolF_ && residueU_ < tolU_) {
            iteration_finish();
            if (adaptive_) {
                // gsALMBase::computeLength (gsALMBase.hpp:105-116): a quotient of two index_t,
                // so an integer division, then clamped to [0.5, 2]
                double fac = (double)(desiredIt_ / num_it_);
                fac = std::min(std::max(fac, 0.5), 2.0);
                arcLength_prev_ = arcLength_;
                arcLength_ = arcLength_ * fac;
            } else {
                arcLength_prev_ = arcLength_;
            }
            return;
        } else if (num_it_ == maxIt_ - 1) {
            throw Fail{ST_NOT_CONVERGED};
        }
    }
}

int ALMGPU::step() {
    try {
        step_impl();
        return ST_SUCCESS;
    } catch (const Fail& f) {
        return f.code;
    }
}

// ------------------------------------------------------------------------------------------
// singular points (gsALMBase.hpp:421-512, 628-852).  The extended system differentiates the
// Jacobian by a forward difference with eps = 1e-8, which cancels to noise unless u_t solves
// K u_t = F to FP64 working accuracy: these solves use FP64 fronts.
// ------------------------------------------------------------------------------------------
void ALMGPU::factor64_at(const double* d_x) {
    if (!S64_) {
        S64_.reset(new MFSolver(P_, 0, 0.0, true));
        for (DevBuf<double>* b : {&V_, &DV_, &dV_, &ut64_, &ub64_, &h1_, &h2_, &Vt_, &Vb_, &W_}) {
            b->alloc(n_);
            b->zero(P_.stream);
        }
        Kv_.alloc(P_.nnz);
    }
    P_.set_displacement(d_x);
    ++n_jac;
    if (S64_->compute_tangent() != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
}

namespace {
double dnorm(const double* x, int n, cudaStream_t s) {
    double d;
    const double* a[1] = {x};
    vec::multidot(1, a, a, n, &d, s);
    return std::sqrt(d);
}
}  // namespace

bool ALMGPU::test_singular_point(bool jacobian) {
    cudaStream_t s = P_.stream;
    if (jacobian)
        KL_CUDA(cudaMemcpyAsync(xjac_.get(), U_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
    // the current Jacobian, in FP64 fronts (gsALMBase.hpp:631-640)
    factor64_at(xjac_.get());
    std::vector<double> ones(n_, 1.0 / std::sqrt((double)n_));
    KL_CUDA(cudaMemcpyAsync(V_.get(), ones.data(), sizeof(double) * n_, cudaMemcpyHostToDevice, s));
    for (int k = 0; k < spTestIt_; ++k) {
        if (S64_->solve(V_.get(), W_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        const double nv = dnorm(W_.get(), n_, s);
        vec::lincomb(1.0 / nv, W_.get(), 0.0, W_.get(), V_.get(), n_, s);
    }
    double dot;
    const double* a[1] = {V_.get()};
    const double* b[1] = {P_.d_F.get()};
    vec::multidot(1, a, b, n_, &dot, s);
    return std::fabs(dot) < spTestTol_;
}

bool ALMGPU::is_bifurcation(bool jacobian) {
    try {
        return test_singular_point(jacobian);
    } catch (const Fail&) {
        return false;
    }
}

void ALMGPU::extended_system_iteration() {
    cudaStream_t s = P_.stream;
    compute_residual();   // R at (U + DU, L + DL)
    vec::lincomb(1.0, U_.get(), 1.0, DU_.get(), x_.get(), n_, s);
    factor64_at(x_.get());
    KL_CUDA(cudaMemcpyAsync(Kv_.get(), P_.d_vals64.get(), sizeof(double) * P_.nnz, cudaMemcpyDeviceToDevice, s));
    if (S64_->solve(P_.d_F.get(), ut64_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
    vec::lincomb(-1.0, R_.get(), 0.0, R_.get(), tmp_.get(), n_, s);
    if (S64_->solve(tmp_.get(), ub64_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
    const double eps = 1e-8;
    vec::lincomb(1.0, V_.get(), 1.0, DV_.get(), W_.get(), n_, s);
    // K_eps at x + eps W (FP64 values only; the factorisation of K stays)
    vec::lincomb(1.0, x_.get(), eps, W_.get(), tmp_.get(), n_, s);
    P_.set_displacement(tmp_.get());
    P_.tangent_f64();
    ++n_jac;
    // h1 = (K_eps u_t - F) / eps,  h2 = K W + (K_eps u_bar + R) / eps
    spmv_vals(P_, P_.d_vals64.get(), ut64_.get(), h1_.get());
    vec::lincomb(1.0 / eps, h1_.get(), -1.0 / eps, P_.d_F.get(), h1_.get(), n_, s);
    spmv_vals(P_, P_.d_vals64.get(), ub64_.get(), h2_.get());
    vec::axpby(1.0 / eps, R_.get(), 1.0 / eps, h2_.get(), n_, s);
    spmv_vals(P_, Kv_.get(), W_.get(), tmp_.get());
    vec::axpby(1.0, tmp_.get(), 1.0, h2_.get(), n_, s);
    vec::lincomb(-1.0, h1_.get(), 0.0, h1_.get(), tmp_.get(), n_, s);
    if (S64_->solve(tmp_.get(), Vt_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
    vec::lincomb(-1.0, h2_.get(), 0.0, h2_.get(), tmp_.get(), n_, s);
    if (S64_->solve(tmp_.get(), Vb_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
    double d[3];
    const double* xs[3] = {W_.get(), W_.get(), W_.get()};
    const double* ys[3] = {W_.get(), Vb_.get(), Vt_.get()};
    vec::multidot(3, xs, ys, n_, d, s);
    const double nW = std::sqrt(d[0]);
    dL_ = -(d[1] / nW + nW - 1.0) / (d[2] / nW);
    vec::lincomb(dL_, ut64_.get(), 1.0, ub64_.get(), dU_.get(), n_, s);
    vec::lincomb(dL_, Vt_.get(), 1.0, Vb_.get(), dV_.get(), n_, s);
}

bool ALMGPU::extended_system_solve(double tol) {
    cudaStream_t s = P_.stream;
    factor64_at(U_.get());
    for (DevBuf<double>* b : {&DV_, &DU_, &dV_, &dU_}) b->zero(s);
    DL_ = dL_ = 0.0;
    for (num_it_ = 0; num_it_ < maxIt_; ++num_it_) {
        extended_system_iteration();
        vec::axpby(1.0, dU_.get(), 1.0, DU_.get(), n_, s);
        DL_ += dL_;
        vec::axpby(1.0, dV_.get(), 1.0, DV_.get(), n_, s);
        vec::lincomb(1.0, U_.get(), 1.0, DU_.get(), x_.get(), n_, s);
        factor64_at(x_.get());
        vec::lincomb(1.0, V_.get(), 1.0, DV_.get(), W_.get(), n_, s);
        spmv_vals(P_, P_.d_vals64.get(), W_.get(), tmp_.get());
        residueKTPhi_ = dnorm(tmp_.get(), n_, s);
        compute_residual();
        compute_residual_norms();
        if (residueKTPhi_ < tol) {
            vec::axpby(1.0, DU_.get(), 1.0, U_.get(), n_, s);
            L_ += DL_;
            return true;
        }
        if (num_it_ == maxIt_ - 1) {
            if (spFail_ == 1) {
                vec::axpby(1.0, DU_.get(), 1.0, U_.get(), n_, s);
                L_ += DL_;
            } else {
                for (DevBuf<double>* b : {&DV_, &DU_, &dV_, &dU_}) b->zero(s);
                DL_ = dL_ = 0.0;
            }
            return false;
        }
    }
    return true;
}

bool ALMGPU::bisection_solve(double tol) {
    cudaStream_t s = P_.stream;
    DevBuf<double> Uold(n_);
    KL_CUDA(cudaMemcpyAsync(Uold.get(), U_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
    double Lold = L_;
    const double dL = arcLength_;
    const bool adaptive = adaptive_;
    adaptive_ = false;
    bool converged = false;
    stability_impl(true, -1e2);
    const double reference = indicator_;
    stability_impl(false, -1e2);
    int64_t fa = negatives_;
    for (int k = 1; k < maxIt_; ++k) {
        KL_CUDA(cudaMemcpyAsync(U_.get(), Uold.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        L_ = Lold;
        const int status = step();
        stability_impl(true, -1e2);
        const int64_t fb = negatives_;
        if (fa == fb && status == ST_SUCCESS) {
            KL_CUDA(cudaMemcpyAsync(Uold.get(), U_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
            Lold = L_;
            fa = fb;
        } else {
            arcLength_ = arcLength_ / 2.0;
        }
        stability_impl(false, -1e2);
        if (std::fabs(indicator_ / reference) < tol) {
            converged = true;
            break;
        }
    }
    arcLength_ = dL;
    adaptive_ = adaptive;
    // null vector of the last Jacobian by inverse iteration (gsALMBase.hpp:820-836)
    factor64_at(xjac_.get());
    std::vector<double> ones(n_, 1.0 / std::sqrt((double)n_));
    KL_CUDA(cudaMemcpyAsync(V_.get(), ones.data(), sizeof(double) * n_, cudaMemcpyHostToDevice, s));
    DevBuf<double> Vold(n_);
    Vold.zero(s);
    for (int k = 0; k < 5; ++k) {
        if (S64_->solve(V_.get(), W_.get(), 1) != ST_SUCCESS) throw Fail{ST_SOLVER_ERROR};
        const double nv = dnorm(W_.get(), n_, s);
        vec::lincomb(1.0 / nv, W_.get(), 0.0, W_.get(), V_.get(), n_, s);
        vec::lincomb(1.0, V_.get(), -1.0, Vold.get(), tmp_.get(), n_, s);
        if (dnorm(tmp_.get(), n_, s) < tolerance_) {
            converged = true;
            break;
        }
        KL_CUDA(cudaMemcpyAsync(Vold.get(), V_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
    }
    return converged;
}

int ALMGPU::compute_singular_point(const double* d_U, double L, bool switch_branch_after, bool jacobian,
                                   bool test_point) {
    try {
        const bool test = test_point ? test_singular_point(jacobian) : true;
        KL_CUDA(cudaMemcpyAsync(U_.get(), d_U, sizeof(double) * n_, cudaMemcpyDeviceToDevice, P_.stream));
        L_ = L;
        if (test) {
            if (!S64_) factor64_at(U_.get());
            if (spTolB_ != 0.0) bisection_solve(spTolB_);
            const bool converged = extended_system_solve(spTolE_);
            if (switch_branch_after && (converged || spFail_ == 1)) switch_branch();
            stability_ = stabilityPrev_;
        }
        return ST_SUCCESS;
    } catch (const Fail& f) {
        return f.code;
    }
}

void ALMGPU::switch_branch() {
    // gsALMBase.hpp:839-852
    cudaStream_t s = P_.stream;
    if (!S64_) return;
    const double nv = dnorm(V_.get(), n_, s);
    vec::lincomb(1.0 / nv, V_.get(), 0.0, V_.get(), V_.get(), n_, s);
    const double xi = dnorm(V_.get(), n_, s) / tau_;
    vec::lincomb(xi, V_.get(), 0.0, V_.get(), DU_.get(), n_, s);
    vec::axpby(1.0, DU_.get(), 1.0, U_.get(), n_, s);
    DLold_ = 0.0;
    DUold_.zero(s);
}

}  // namespace klsa
