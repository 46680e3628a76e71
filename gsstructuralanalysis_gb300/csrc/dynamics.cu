// dynamics.cu -- gsDynamicSolvers time integrators on the device (see dynamics.h).
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "dynamics.h"
#include "eigen.h"

namespace klsa {

namespace {

// out = a X + b Y + c Z over nnz matrix values (Y or Z may be null)
__global__ void vals_combine_kernel(int64_t nnz, double a, const double* __restrict__ X, double b,
                                    const double* __restrict__ Y, double c, const double* __restrict__ Z,
                                    double* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnz) return;
    double v = a * X[i];
    if (Y) v += b * Y[i];
    if (Z) v += c * Z[i];
    out[i] = v;
}

constexpr int NW = 16;   // work vectors

}  // namespace

DynamicGPU::DynamicGPU(Problem& P, Method m, bool nonlinear, const Options& opt)
    : P_(P), method_(m), nl_(nonlinear), opt_(opt) {
    // gsDynamicBase.hpp:19-33 and the integrators' defaultOptions()
    dt_ = opt.real("DT", 1e-2);
    maxIt_ = (int)opt.integer("MaxIter", 100);
    tolF_ = opt.real("TolF", 1e-3);
    tolU_ = opt.real("TolU", 1e-6);
    quasi_ = opt.integer("Quasi", 0) != 0;
    quasiIt_ = (int)opt.integer("QuasiIterations", 1);
    alpha_ = opt.real("alpha", 0.25);
    delta_ = opt.real("delta", 0.5);
    gamma_ = opt.real("gamma", m == Wilson ? 1.4 : 0.5);
    cM_ = opt.real("DampingMass", 0.0);
    cK_ = opt.real("DampingStiffness", 0.0);
    fp64_ = opt.integer("FrontPrecision", 64) == 64;
    std::string solver = opt.str("Solver", "SimplicialLDLT");
    if (solver != "SimplicialLDLT" && solver != "SimplicialLLT" && solver != "LDLT" && solver != "SparseLU")
        throw std::invalid_argument("time integrators need a direct solver (SimplicialLDLT), got " + solver);
    if (quasiIt_ < 1) quasiIt_ = 1;
    if (m == Bathe && (gamma_ <= 0.0 || gamma_ >= 1.0)) throw std::invalid_argument("Bathe: gamma must lie in (0, 1)");
    if (m == Wilson && gamma_ == 0.0) throw std::invalid_argument("Wilson: gamma must be nonzero");

    S_.reset(new MFSolver(P_, fp64_ ? 0 : (int)opt.integer("Refinement", 12), opt.real("RefineTol", 1e-14), fp64_));
    const int n = P_.nfree;
    const int64_t nnz = P_.nnz;
    U_.alloc(n); V_.alloc(n); A_.alloc(n);
    U_.zero(P_.stream); V_.zero(P_.stream); A_.zero(P_.stream);
    W_.alloc((size_t)NW * n);
    fint_.alloc(n);
    lhs_.alloc(nnz);
    // constant matrices: consistent mass, linear stiffness, Rayleigh damping
    P_.mass_f64();
    M_.alloc(nnz);
    KL_CUDA(cudaMemcpyAsync(M_.get(), P_.d_vals64.get(), sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P_.stream));
    if (!nl_ || cK_ != 0.0) {
        KL_.alloc(nnz);
        double* z = w(0);
        KL_CUDA(cudaMemsetAsync(z, 0, sizeof(double) * n, P_.stream));
        P_.set_displacement(z);
        P_.tangent_f64();
        KL_CUDA(cudaMemcpyAsync(KL_.get(), P_.d_vals64.get(), sizeof(double) * nnz, cudaMemcpyDeviceToDevice,
                                P_.stream));
    }
    has_damping_ = cM_ != 0.0 || cK_ != 0.0;
    if (has_damping_) {
        C_.alloc(nnz);
        vals_combine_kernel<<<ceil_div(nnz, 256), 256, 0, P_.stream>>>(nnz, cM_, M_.get(), cK_, KL_.get(), 0.0,
                                                                        nullptr, C_.get());
        count_launch();
    }
    if (nl_) K_.alloc(nnz);
    KL_CUDA(cudaStreamSynchronize(P_.stream));
}

double* DynamicGPU::w(int i) { return W_.get() + (size_t)i * P_.nfree; }

void DynamicGPU::set_load_table(const std::vector<double>& t, const std::vector<double>& f) {
    if (t.size() != f.size()) throw std::invalid_argument("load table: times and factors differ in length");
    for (size_t i = 1; i < t.size(); ++i)
        if (!(t[i] >= t[i - 1])) throw std::invalid_argument("load table: times must be non-decreasing");
    lt_ = t;
    lf_ = f;
}

double DynamicGPU::load_factor(double t) const {
    if (lt_.empty()) return 1.0;
    if (t <= lt_.front()) return lf_.front();
    if (t >= lt_.back()) return lf_.back();
    size_t j = std::upper_bound(lt_.begin(), lt_.end(), t) - lt_.begin();   // lt_[j-1] <= t < lt_[j]
    double a = (t - lt_[j - 1]) / (lt_[j] - lt_[j - 1]);
    return lf_[j - 1] + a * (lf_[j] - lf_[j - 1]);
}

// ---- callbacks ------------------------------------------------------------------------------
void DynamicGPU::residual(const double* U, double t, double* R) {
    P_.set_displacement(U);
    P_.internal_force(fint_.get());
    vec::lincomb(load_factor(t), P_.d_F.get(), -1.0, fint_.get(), R, P_.nfree, P_.stream);
}

void DynamicGPU::force(double t, double* F) {
    vec::lincomb(load_factor(t), P_.d_F.get(), 0.0, P_.d_F.get(), F, P_.nfree, P_.stream);
}

void DynamicGPU::tangent(const double* U) {
    if (!nl_) return;   // the linear integrators use the constant stiffness K_L
    P_.set_displacement(U);
    P_.tangent_f64();
    KL_CUDA(cudaMemcpyAsync(K_.get(), P_.d_vals64.get(), sizeof(double) * P_.nnz, cudaMemcpyDeviceToDevice,
                            P_.stream));
}

void DynamicGPU::mass_apply(const double* x, double* y) { spmv_vals(P_, M_.get(), x, y); }

void DynamicGPU::damp_apply(const double* x, double* y) {
    if (has_damping_) spmv_vals(P_, C_.get(), x, y);
    else KL_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * P_.nfree, P_.stream));
}

void DynamicGPU::stiff_apply(const double* x, double* y) { spmv_vals(P_, nl_ ? K_.get() : KL_.get(), x, y); }

uint64_t DynamicGPU::generation() { return fp64_ ? P_.solver64().generation() : P_.solver().generation(); }

int DynamicGPU::factor(double cM, double cC, double cK, bool cacheable) {
    // the fronts are shared with every other solver of the problem: reuse them only when no one
    // has factorised since
    if (cacheable && factored_ == 2 && gen_ == generation() && fkey_[0] == cM && fkey_[1] == cC && fkey_[2] == cK)
        return ST_SUCCESS;
    const int64_t nnz = P_.nnz;
    vals_combine_kernel<<<ceil_div(nnz, 256), 256, 0, P_.stream>>>(nnz, cM, M_.get(), cC, has_damping_ ? C_.get() : nullptr,
                                                                    cK, nl_ ? K_.get() : KL_.get(), lhs_.get());
    count_launch();
    KL_CUDA(cudaMemcpyAsync(P_.d_vals64.get(), lhs_.get(), sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P_.stream));
    cur_ = lhs_.get();
    factored_ = 0;
    if (S_->factor_current(true) != ST_SUCCESS) return ST_SOLVER_ERROR;
    factored_ = cacheable ? 2 : 3;
    gen_ = generation();
    fkey_[0] = cM; fkey_[1] = cC; fkey_[2] = cK;
    return ST_SUCCESS;
}

int DynamicGPU::factor_mass() {
    if (factored_ == 1 && gen_ == generation()) return ST_SUCCESS;
    KL_CUDA(cudaMemcpyAsync(P_.d_vals64.get(), M_.get(), sizeof(double) * P_.nnz, cudaMemcpyDeviceToDevice, P_.stream));
    cur_ = M_.get();
    factored_ = 0;
    if (S_->factor_current(true) != ST_SUCCESS) return ST_SOLVER_ERROR;
    factored_ = 1;
    gen_ = generation();
    return ST_SUCCESS;
}

int DynamicGPU::solve(const double* b, double* x) {
    // FP32 fronts refine against the FP64 values in the problem's value array, which the tangent
    // assembly reuses: put the factorised matrix back first
    if (!fp64_)
        KL_CUDA(cudaMemcpyAsync(P_.d_vals64.get(), cur_, sizeof(double) * P_.nnz, cudaMemcpyDeviceToDevice, P_.stream));
    return S_->solve(b, x, 1) == ST_SUCCESS ? ST_SUCCESS : ST_SOLVER_ERROR;
}

double DynamicGPU::norm(const double* x) {
    double d = 0.0;
    vec::multidot(1, &x, &x, P_.nfree, &d, P_.stream);
    return std::sqrt(d);
}

double DynamicGPU::norm2(const double* x, const double* y) {
    double d[2] = {0.0, 0.0};
    const double* xs[2] = {x, y};
    vec::multidot(2, xs, xs, P_.nfree, d, P_.stream);
    return std::sqrt(d[0] + d[1]);
}

bool DynamicGPU::bad(double nrm) { return std::isinf(nrm) || std::isnan(nrm); }

void DynamicGPU::copy(const double* x, double* y) {
    KL_CUDA(cudaMemcpyAsync(y, x, sizeof(double) * P_.nfree, cudaMemcpyDeviceToDevice, P_.stream));
}

void DynamicGPU::axpy(double a, const double* x, double* y) { vec::axpby(a, x, 1.0, y, P_.nfree, P_.stream); }

void DynamicGPU::lin(double a, const double* x, double b, const double* y, double* z) {
    vec::lincomb(a, x, b, y, z, P_.nfree, P_.stream);
}

// ---- Newmark (gsDynamicNewmark.hpp:30-145) -----------------------------------------------------
// Work vectors 0..7.
int DynamicGPU::newmark(double t, double dt, double* U, double* V, double* A) {
    const double al = alpha_, de = delta_;
    double *Uold = w(0), *Vold = w(1), *Aold = w(2), *F = w(3), *r = w(4), *s = w(5), *rhs = w(6), *dA = w(7);
    copy(U, Uold); copy(V, Vold); copy(A, Aold);
    if (!nl_) {
        force(t + dt, F);
        lin(1.0, Uold, dt, Vold, U);
        axpy((0.5 - al) * dt * dt, Aold, U);
        lin(1.0, Vold, (1 - de) * dt, Aold, V);
        tangent(U);
        if (factor(1.0, de * dt, dt * dt * al, true) != ST_SUCCESS) return ST_SOLVER_ERROR;
        stiff_apply(U, r);
        damp_apply(V, s);
        lin(1.0, F, -1.0, r, rhs);
        axpy(-1.0, s, rhs);
        if (solve(rhs, A) != ST_SUCCESS) return ST_SOLVER_ERROR;
        axpy(de * dt, A, V);
        axpy(al * dt * dt, A, U);
        iterations_ = 1;
        return bad(norm(U)) ? ST_NOT_CONVERGED : ST_SUCCESS;
    }
    KL_CUDA(cudaMemsetAsync(A, 0, sizeof(double) * P_.nfree, P_.stream));
    lin(1.0, Uold, dt, Vold, U);
    axpy((0.5 - al) * dt * dt, Aold, U);
    lin(1.0, Vold, (1 - de) * dt, Aold, V);
    auto make_rhs = [&]() {   // rhs = R(U, t+dt) - C V - M A
        residual(U, t + dt, F);
        damp_apply(V, r);
        mass_apply(A, s);
        lin(1.0, F, -1.0, r, rhs);
        axpy(-1.0, s, rhs);
    };
    make_rhs();
    double r0 = norm(rhs);
    if (r0 == 0.0) r0 = 1.0;
    iterations_ = 0;
    for (int it = 0; it < maxIt_; ++it) {
        if (!quasi_ || it == 0 || it % quasiIt_ == 0) tangent(U);
        if (factor(1.0, de * dt, dt * dt * al, false) != ST_SUCCESS) return ST_SOLVER_ERROR;
        if (solve(rhs, dA) != ST_SUCCESS) return ST_SOLVER_ERROR;
        axpy(1.0, dA, A);
        axpy(de * dt, dA, V);
        axpy(al * dt * dt, dA, U);
        double An = norm(A), dAn = norm(dA);
        double upd = An != 0.0 ? dAn / An : dAn;
        make_rhs();
        double res = norm(rhs) / r0;
        iterations_ = it + 1;
        if (upd < tolU_ && res < tolF_) return ST_SUCCESS;
    }
    return ST_NOT_CONVERGED;
}

// ---- Bathe (gsDynamicBathe.hpp:30-163) -------------------------------------------------------
int DynamicGPU::bathe(double t, double dt) {
    const double g = gamma_;
    double *Uold = w(8), *Vold = w(9), *Us = w(10), *Vs = w(11), *As = w(12), *R = w(13), *tmp = w(14);
    copy(U_.get(), Uold); copy(V_.get(), Vold);
    copy(U_.get(), Us); copy(V_.get(), Vs); copy(A_.get(), As);
    int its = 0;
    newmark(t, g * dt, Us, Vs, As);   // stage 1 (its status is not used, as in the reference)
    its += iterations_;
    const double c1 = (1 - g) / (g * dt), c2 = -1.0 / ((1 - g) * g * dt), c3 = (2 - g) / ((1 - g) * dt);
    double *a = w(0), *b = w(1), *rhs = w(2), *dU = w(3), *tmp2 = w(4);
    // rhs = R - M (c1 Vold + c2 Vs + c1 c3 Uold + c3 c2 Us + c3^2 U) - C (c1 Uold + c2 Us + c3 U),
    // without the U terms in the linear variant
    auto make_rhs = [&](const double* Rv, const double* U, bool with_u) {
        lin(c1, Vold, c2, Vs, tmp);
        axpy(c1 * c3, Uold, tmp);
        axpy(c3 * c2, Us, tmp);
        if (with_u) axpy(c3 * c3, U, tmp);
        mass_apply(tmp, a);
        lin(c1, Uold, c2, Us, tmp2);
        if (with_u) axpy(c3, U, tmp2);
        damp_apply(tmp2, b);
        lin(1.0, Rv, -1.0, a, rhs);
        axpy(-1.0, b, rhs);
    };
    auto finish = [&]() {
        lin(c1, Uold, c2, Us, V_.get());
        axpy(c3, U_.get(), V_.get());
        lin(c1, Vold, c2, Vs, A_.get());
        axpy(c3, V_.get(), A_.get());
    };
    if (!nl_) {
        force(t + dt, R);
        tangent(Uold);
        if (factor(c3 * c3, c3, 1.0, true) != ST_SUCCESS) return ST_SOLVER_ERROR;
        make_rhs(R, nullptr, false);
        if (solve(rhs, U_.get()) != ST_SUCCESS) return ST_SOLVER_ERROR;
        finish();
        iterations_ = its + 1;
        return bad(norm(U_.get())) ? ST_NOT_CONVERGED : ST_SUCCESS;
    }
    residual(Uold, t + dt, R);           // evaluated before U is reset to the stage-1 state
    copy(Us, U_.get()); copy(Vs, V_.get()); copy(As, A_.get());
    make_rhs(R, U_.get(), true);
    double r0 = norm(rhs);
    if (r0 == 0.0) r0 = 1.0;
    for (int it = 0; it < maxIt_; ++it) {
        if (!quasi_ || it == 0 || it % quasiIt_ == 0) tangent(U_.get());
        if (factor(c3 * c3, c3, 1.0, false) != ST_SUCCESS) return ST_SOLVER_ERROR;
        if (solve(rhs, dU) != ST_SUCCESS) return ST_SOLVER_ERROR;
        axpy(1.0, dU, U_.get());
        residual(U_.get(), t + dt, R);
        make_rhs(R, U_.get(), true);
        double res = norm(rhs) / r0;
        double upd = norm(dU) / norm(U_.get());
        iterations_ = its + it + 1;
        if (upd < tolU_ && res < tolF_) {
            finish();
            return ST_SUCCESS;
        }
    }
    finish();
    return ST_NOT_CONVERGED;
}

// ---- Wilson (gsDynamicWilson.hpp:30-82) ------------------------------------------------------
int DynamicGPU::wilson(double t, double dt) {
    const double al = alpha_, de = delta_, g = gamma_;
    double *Uold = w(8), *Vold = w(9), *Aold = w(10), *Ut = w(11), *Vt = w(12), *At = w(13);
    copy(U_.get(), Uold); copy(V_.get(), Vold); copy(A_.get(), Aold);
    copy(U_.get(), Ut); copy(V_.get(), Vt); copy(A_.get(), At);
    newmark(t, g * dt, Ut, Vt, At);   // its status is not used, as in the reference
    lin(1.0 - 1.0 / g, Aold, 1.0 / g, At, A_.get());
    if (!nl_) {
        lin(1.0, Vold, de * dt, A_.get(), V_.get());
        lin(1.0, Uold, al * dt * dt, A_.get(), U_.get());
    } else {
        lin(1.0, Uold, dt, Vold, U_.get());
        axpy((0.5 - al) * dt * dt, Aold, U_.get());
        axpy(al * dt * dt, A_.get(), U_.get());
        lin(1.0, Vold, (1 - de) * dt, Aold, V_.get());
        axpy(de * dt, A_.get(), V_.get());
    }
    return ST_SUCCESS;
}

// ---- explicit Euler (gsDynamicExplicitEuler.hpp:53-131) ----------------------------------------
int DynamicGPU::explicit_euler(double t, double dt) {
    double *Uold = w(8), *Vold = w(9), *f = w(0), *cv = w(1), *b = w(2), *acc = w(3), *ku = w(4);
    copy(U_.get(), Uold); copy(V_.get(), Vold);
    damp_apply(Vold, cv);
    if (!nl_) {
        force(t, f);
        stiff_apply(Uold, ku);
        lin(1.0, f, -1.0, ku, b);
        axpy(-1.0, cv, b);
    } else {
        residual(Uold, t, f);
        lin(-1.0, f, -1.0, cv, b);      // M^-1 (-R - C V), the reference's sign
    }
    if (factor_mass() != ST_SUCCESS) return ST_SOLVER_ERROR;
    if (solve(b, acc) != ST_SUCCESS) return ST_SOLVER_ERROR;
    lin(1.0, Uold, dt, Vold, U_.get());
    lin(1.0, Vold, dt, acc, V_.get());
    iterations_ = 1;
    return bad(norm2(U_.get(), V_.get())) ? ST_NOT_CONVERGED : ST_SUCCESS;
}

// ---- implicit Euler (gsDynamicImplicitEuler.hpp:24-163) ----------------------------------------
// The 2x2 block system [[I, -dt I], [dt K, M + dt C]] (solved by GMRES in the reference) is solved
// exactly by eliminating the displacement block: (M + dt C + dt^2 K) dV = -r_V + dt K r_U.
int DynamicGPU::implicit_euler(double t, double dt) {
    double *Uold = w(8), *Vold = w(9), *R = w(10), *dU = w(11);
    double *rU = w(0), *rV = w(1), *tmp = w(2), *mv = w(3), *cv = w(4), *b = w(5), *kr = w(6), *dV = w(7);
    copy(U_.get(), Uold); copy(V_.get(), Vold);
    if (!nl_) {
        force(t + dt, R);
        tangent(Uold);
        if (factor(1.0, dt, dt * dt, true) != ST_SUCCESS) return ST_SOLVER_ERROR;
        mass_apply(Vold, mv);
        stiff_apply(Uold, kr);
        lin(dt, R, 1.0, mv, b);
        axpy(-dt, kr, b);
        if (solve(b, V_.get()) != ST_SUCCESS) return ST_SOLVER_ERROR;
        lin(1.0, Uold, dt, V_.get(), U_.get());
        iterations_ = 1;
        return ST_SUCCESS;
    }
    residual(U_.get(), t + dt, R);
    damp_apply(V_.get(), cv);
    lin(-dt, V_.get(), 0.0, V_.get(), rU);
    lin(dt, cv, -dt, R, rV);
    double r0 = norm2(rU, rV);
    if (r0 == 0.0) r0 = 1.0;
    for (int it = 0; it < maxIt_; ++it) {
        if (!quasi_ || it == 0 || it % quasiIt_ == 0) tangent(U_.get());
        // r_U = U - Uold - dt V,  r_V = M (V - Vold) + dt C V - dt R
        lin(1.0, U_.get(), -1.0, Uold, rU);
        axpy(-dt, V_.get(), rU);
        lin(1.0, V_.get(), -1.0, Vold, tmp);
        mass_apply(tmp, mv);
        damp_apply(V_.get(), cv);
        lin(1.0, mv, dt, cv, rV);
        axpy(-dt, R, rV);
        if (factor(1.0, dt, dt * dt, false) != ST_SUCCESS) return ST_SOLVER_ERROR;
        stiff_apply(rU, kr);
        lin(-1.0, rV, dt, kr, b);
        if (solve(b, dV) != ST_SUCCESS) return ST_SOLVER_ERROR;
        lin(dt, dV, -1.0, rU, dU);
        axpy(1.0, dU, U_.get());
        axpy(1.0, dV, V_.get());
        double sn = norm2(U_.get(), V_.get()), dn = norm2(dU, dV);
        double upd = sn != 0.0 ? dn / sn : dn;
        residual(U_.get(), t, R);          // the reference evaluates it at t here
        double res = norm2(rU, rV) / r0;   // the residual of the iterate before this update
        iterations_ = it + 1;
        if (upd < tolU_ && res < tolF_) return ST_SUCCESS;
    }
    return ST_NOT_CONVERGED;
}

// ---- RK4 (gsDynamicRK4.hpp:18-150) ------------------------------------------------------------
int DynamicGPU::rk4(double t, double dt) {
    double *Uold = w(8), *Vold = w(9), *k1v = w(10), *k2u = w(11), *k2v = w(12), *k3u = w(13), *k3v = w(14),
           *k4v = w(15), *Ut = w(4), *Vt = w(5);
    copy(U_.get(), Uold); copy(V_.get(), Vold);
    if (factor_mass() != ST_SUCCESS) return ST_SOLVER_ERROR;
    // out = M^-1 (Fext(tx) - K Ux - C Vx)  or  M^-1 (R(Ux, tx) - C Vx)
    auto acc = [&](const double* Ux, const double* Vx, double tx, double* out) -> int {
        double *f = w(0), *ku = w(1), *cv = w(2), *b = w(3);
        damp_apply(Vx, cv);
        if (!nl_) {
            force(tx, f);
            stiff_apply(Ux, ku);
            lin(1.0, f, -1.0, ku, b);
            axpy(-1.0, cv, b);
        } else {
            residual(Ux, tx, f);
            lin(1.0, f, -1.0, cv, b);
        }
        return solve(b, out);
    };
    if (acc(Uold, Vold, t, k1v) != ST_SUCCESS) return ST_SOLVER_ERROR;
    lin(1.0, Uold, dt / 2, Vold, Ut);
    lin(1.0, Vold, dt / 2, k1v, Vt);
    copy(Vt, k2u);
    if (acc(Ut, Vt, t + dt / 2, k2v) != ST_SUCCESS) return ST_SOLVER_ERROR;
    lin(1.0, Uold, dt / 2, k2u, Ut);
    lin(1.0, Vold, dt / 2, k2v, Vt);
    copy(Vt, k3u);
    if (acc(Ut, Vt, t + dt / 2, k3v) != ST_SUCCESS) return ST_SOLVER_ERROR;
    lin(1.0, Uold, dt, k3u, Ut);
    lin(1.0, Vold, dt, k3v, Vt);                 // Vt is k4u from here on
    if (acc(Ut, Vt, t + dt, k4v) != ST_SUCCESS) return ST_SOLVER_ERROR;
    const double h = dt / 6.0;
    lin(1.0, Uold, h, Vold, U_.get());
    axpy(2 * h, k2u, U_.get());
    axpy(2 * h, k3u, U_.get());
    axpy(h, Vt, U_.get());
    lin(1.0, Vold, h, k1v, V_.get());
    axpy(2 * h, k2v, V_.get());
    axpy(2 * h, k3v, V_.get());
    axpy(h, k4v, V_.get());
    iterations_ = 1;
    return bad(norm2(U_.get(), V_.get())) ? ST_NOT_CONVERGED : ST_SUCCESS;
}

int DynamicGPU::step(double dt) {
    int st = ST_OTHER_ERROR;
    switch (method_) {
        case Newmark: st = newmark(time_, dt, U_.get(), V_.get(), A_.get()); break;
        case Bathe: st = bathe(time_, dt); break;
        case Wilson: st = wilson(time_, dt); break;
        case ExplicitEuler: st = explicit_euler(time_, dt); break;
        case ImplicitEuler: st = implicit_euler(time_, dt); break;
        case RK4: st = rk4(time_, dt); break;
    }
    time_ += dt;
    return st;
}

}  // namespace klsa
