// CPU oracle built from the reference's OWN solver headers (test infrastructure only).
//
// gsStaticNewton, gsALMCrisfield, gsALMRiks, gsALMLoadControl, gsALMConsistentCrisfield,
// gsAPALM (the build without MPI: serialSolve, the one-process parallelSolve and solve),
// gsModalSolver, gsBucklingSolver and the time integrators gsDynamicNewmark, gsDynamicBathe,
// gsDynamicWilson, gsDynamicExplicitEuler, gsDynamicImplicitEuler and gsDynamicRK4 are compiled
// unchanged from the reference tree (src/gsStaticSolvers, src/gsALMSolvers, src/gsEigenSolvers,
// src/gsDynamicSolvers) against the test-only stand-in of
// gismo's linear algebra and option list in oracle/refshim/.  The operators they call -- the
// reference's Jacobian_t, Residual_t and ALResidual_t callbacks
// (src/gsStructuralAnalysisTools/gsStructuralAnalysisTypes.h:58-93) -- are C function pointers
// supplied by the caller (the tests bind them to the FP64 KL-shell oracle assembler).  The
// solver logic that runs is therefore the reference's own; only the matrix arithmetic under it
// is the stand-in's.  Built by oracle/Makefile into oracle/_ref/ (never shipped, never linked by
// the product).
#include <cstdint>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include <gsStructuralAnalysis/src/gsALMSolvers/gsALMConsistentCrisfield.h>
// gsAPALMDataContainer.h names gsAPALMData without including it (gismo's module header
// includes both); the data header comes first here for the same reason
#include <gsStructuralAnalysis/src/gsALMSolvers/gsAPALMData.h>
#include <gsStructuralAnalysis/src/gsALMSolvers/gsAPALM.h>
#include <gsStructuralAnalysis/src/gsALMSolvers/gsALMCrisfield.h>
#include <gsStructuralAnalysis/src/gsALMSolvers/gsALMLoadControl.h>
#include <gsStructuralAnalysis/src/gsALMSolvers/gsALMRiks.h>
#include <gsStructuralAnalysis/src/gsEigenSolvers/gsBucklingSolver.h>
#include <gsStructuralAnalysis/src/gsEigenSolvers/gsModalSolver.h>
#include <gsStructuralAnalysis/src/gsStaticSolvers/gsStaticNewton.h>
#include <gsStructuralAnalysis/src/gsDynamicSolvers/gsDynamicBathe.h>
#include <gsStructuralAnalysis/src/gsDynamicSolvers/gsDynamicExplicitEuler.h>
#include <gsStructuralAnalysis/src/gsDynamicSolvers/gsDynamicImplicitEuler.h>
#include <gsStructuralAnalysis/src/gsDynamicSolvers/gsDynamicNewmark.h>
#include <gsStructuralAnalysis/src/gsDynamicSolvers/gsDynamicRK4.h>
#include <gsStructuralAnalysis/src/gsDynamicSolvers/gsDynamicWilson.h>

using namespace gismo;

extern "C" {
// x: free-dof vector; vals: the Jacobian's values in the problem's fixed CSR pattern
typedef int (*refh_jac_fn)(const double* x, double* vals);
// Fint(x) - lambda F  (ALResidual_t)
typedef int (*refh_alres_fn)(const double* x, double lambda, double* R);
// F - Fint(x)  (Residual_t)
typedef int (*refh_res_fn)(const double* x, double* R);
// time-dependent operators of the integrators: x may be null (mass, stiffness, force)
typedef int (*refh_tmat_fn)(const double* x, double t, double* vals);
typedef int (*refh_tvec_fn)(const double* x, double t, double* out);
}

namespace {

thread_local std::string g_err;

struct RefProblem {
    index_t n = 0;
    std::vector<int64_t> rowptr;
    std::vector<int32_t> cols;
    refh_jac_fn jac = nullptr;
    refh_alres_fn alres = nullptr;
    refh_res_fn res = nullptr;
    gsVector<real_t> F;
    gsSparseMatrix<real_t> KL;        // Jacobian at zero (gsStaticNewton keeps a reference)

    bool jacobian(const gsVector<real_t>& x, gsSparseMatrix<real_t>& K) const {
        std::vector<double> v(cols.size());
        if (jac(x.data(), v.data()) != 0) return false;
        K = gsSparseMatrix<real_t>(n, n);
        for (index_t i = 0; i < n; ++i)
            for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) K(i, cols[k]) = v[k];
        return true;
    }
};

// "key=t:value;..." with t in i (int), r (real), b (switch), s (string)
void apply_options(gsOptionList& o, const char* spec) {
    if (!spec) return;
    std::stringstream ss(spec);
    std::string item;
    while (std::getline(ss, item, ';')) {
        if (item.empty()) continue;
        const size_t eq = item.find('='), colon = item.find(':', eq);
        if (eq == std::string::npos || colon == std::string::npos) throw std::runtime_error("bad option " + item);
        const std::string key = item.substr(0, eq), type = item.substr(eq + 1, colon - eq - 1),
                          val = item.substr(colon + 1);
        if (type == "i") o.addInt(key, "", std::stoi(val));
        else if (type == "r") o.addReal(key, "", std::stod(val));
        else if (type == "b") o.addSwitch(key, "", val == "1" || val == "true");
        else if (type == "s") o.addString(key, "", val);
        else throw std::runtime_error("bad option type " + item);
    }
}

template <class F>
int guard(F&& f) {
    try {
        return f();
    } catch (const std::exception& e) {
        g_err = e.what();
    } catch (int) {                 // the integrators throw 2 when an operator callback fails
        g_err = "operator failed";
    } catch (...) {
        g_err = "unknown error";
    }
    return -1;
}

struct RefALM {
    RefProblem* P;
    std::unique_ptr<gsALMBase<real_t>> alm;
};

struct RefNewton {
    RefProblem* P;
    std::unique_ptr<gsStaticNewton<real_t>> N;
};

// gsAPALM with read access to its flat solutions per branch (protected members)
struct HarnessAPALM : public gsAPALM<real_t> {
    HarnessAPALM(gsALMBase<real_t>* alm, const gsAPALMData<real_t, solution_t>& data) : gsAPALM<real_t>(alm, data) {}
    size_t branches() const { return m_solutions.size(); }
};

struct RefAPALM {
    RefALM* A;
    std::unique_ptr<HarnessAPALM> P;
};

struct RefDyn {
    index_t n = 0;
    std::vector<int64_t> rowptr;
    std::vector<int32_t> cols;
    refh_tmat_fn mass = nullptr, damping = nullptr, jac = nullptr;
    refh_tvec_fn vec = nullptr;
    std::unique_ptr<gsDynamicBase<real_t>> D;

    bool matrix(refh_tmat_fn f, const double* x, double t, gsSparseMatrix<real_t>& K) const {
        std::vector<double> v(cols.size());
        if (f(x, t, v.data()) != 0) return false;
        K = gsSparseMatrix<real_t>(n, n);
        for (index_t i = 0; i < n; ++i)
            for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) K(i, cols[k]) = v[k];
        return true;
    }
    bool vector(const double* x, double t, gsVector<real_t>& r) const {
        r = gsVector<real_t>(n);
        return vec(x, t, r.data()) == 0;
    }
};

// One integrator of the reference with the linear constructor (Mass_t, Damping_t, Stiffness_t,
// TForce_t) or the nonlinear one (Mass_t, Damping_t, Jacobian_t, TResidual_t), as
// gsDynamicBase.h:58-130 defines them.
template <template <class, bool> class Integrator>
gsDynamicBase<real_t>* make_dynamic(RefDyn* D, bool nonlinear) {
    typename gsStructuralAnalysisOps<real_t>::Mass_t M = [D](gsSparseMatrix<real_t>& m) {
        return D->matrix(D->mass, nullptr, 0.0, m);
    };
    typename gsStructuralAnalysisOps<real_t>::Damping_t C = [D](gsVector<real_t> const& x, gsSparseMatrix<real_t>& m) {
        return D->matrix(D->damping, x.data(), 0.0, m);
    };
    if (!nonlinear) {
        typename gsStructuralAnalysisOps<real_t>::Stiffness_t K = [D](gsSparseMatrix<real_t>& m) {
            return D->matrix(D->jac, nullptr, 0.0, m);
        };
        typename gsStructuralAnalysisOps<real_t>::TForce_t F = [D](const real_t t, gsVector<real_t>& r) {
            return D->vector(nullptr, t, r);
        };
        return new Integrator<real_t, false>(M, C, K, F);
    }
    typename gsStructuralAnalysisOps<real_t>::Jacobian_t J = [D](gsVector<real_t> const& x, gsSparseMatrix<real_t>& m) {
        return D->matrix(D->jac, x.data(), 0.0, m);
    };
    typename gsStructuralAnalysisOps<real_t>::TResidual_t R = [D](gsVector<real_t> const& x, const real_t t,
                                                                  gsVector<real_t>& r) {
        return D->vector(x.data(), t, r);
    };
    return new Integrator<real_t, true>(M, C, J, R);
}

}  // namespace

extern "C" {

const char* refh_last_error(void) { return g_err.c_str(); }

void* refh_problem_create(int n, int64_t nnz, const int64_t* rowptr, const int32_t* cols, refh_jac_fn jac,
                          refh_alres_fn alres, refh_res_fn res, const double* F) {
    RefProblem* P = new RefProblem();
    P->n = n;
    P->rowptr.assign(rowptr, rowptr + n + 1);
    P->cols.assign(cols, cols + nnz);
    P->jac = jac;
    P->alres = alres;
    P->res = res;
    P->F = gsVector<real_t>(n);
    std::memcpy(P->F.data(), F, sizeof(double) * n);
    if (!P->jacobian(gsVector<real_t>(n), P->KL)) {
        g_err = "Jacobian callback failed at zero";
        delete P;
        return nullptr;
    }
    return P;
}
void refh_problem_destroy(void* p) { delete static_cast<RefProblem*>(p); }

// ---- arc-length methods (gsALMBase and its subclasses) ----------------------------------------
void* refh_alm_create(void* prob, const char* method, const char* options) {
    RefProblem* P = static_cast<RefProblem*>(prob);
    RefALM* A = nullptr;
    int st = guard([&] {
        typename gsStructuralAnalysisOps<real_t>::Jacobian_t J = [P](gsVector<real_t> const& x, gsSparseMatrix<real_t>& m) {
            return P->jacobian(x, m);
        };
        typename gsStructuralAnalysisOps<real_t>::ALResidual_t R = [P](gsVector<real_t> const& x, real_t lam,
                                                                       gsVector<real_t>& r) {
            r = gsVector<real_t>(P->n);
            return P->alres(x.data(), lam, r.data()) == 0;
        };
        std::unique_ptr<gsALMBase<real_t>> alm;
        const std::string m(method);
        if (m == "Crisfield") alm.reset(new gsALMCrisfield<real_t>(J, R, P->F));
        else if (m == "Riks") alm.reset(new gsALMRiks<real_t>(J, R, P->F));
        else if (m == "LoadControl") alm.reset(new gsALMLoadControl<real_t>(J, R, P->F));
        else if (m == "ConsistentCrisfield") alm.reset(new gsALMConsistentCrisfield<real_t>(J, R, P->F));
        else throw std::runtime_error("unknown method " + m);
        gsOptionList o;
        apply_options(o, options);
        alm->setOptions(o);
        A = new RefALM{P, std::move(alm)};
        return 0;
    });
    return st == 0 ? A : nullptr;
}
void refh_alm_destroy(void* a) { delete static_cast<RefALM*>(a); }

int refh_alm_initialize(void* a, int stability) {
    return guard([&] {
        static_cast<RefALM*>(a)->alm->initialize(stability != 0);
        return 0;
    });
}
int refh_alm_step(void* a) {
    return guard([&] { return (int)static_cast<RefALM*>(a)->alm->step(); });
}
int refh_alm_solution(void* a, double* U, double* L) {
    return guard([&] {
        RefALM* A = static_cast<RefALM*>(a);
        const gsVector<real_t>& u = A->alm->solutionU();
        std::memcpy(U, u.data(), sizeof(double) * u.rows());
        *L = A->alm->solutionL();
        return 0;
    });
}
int refh_alm_set_initial_guess(void* a, const double* U, double L) {
    return guard([&] {
        RefALM* A = static_cast<RefALM*>(a);
        gsVector<real_t> u(A->P->n);
        std::memcpy(u.data(), U, sizeof(double) * A->P->n);
        A->alm->setInitialGuess(u, L);
        return 0;
    });
}
int refh_alm_set_solution(void* a, const double* U, double L) {
    return guard([&] {
        RefALM* A = static_cast<RefALM*>(a);
        gsVector<real_t> u(A->P->n);
        std::memcpy(u.data(), U, sizeof(double) * A->P->n);
        A->alm->setSolution(u, L);
        return 0;
    });
}
int refh_alm_set_length(void* a, double length) {
    return guard([&] {
        static_cast<RefALM*>(a)->alm->setLength(length);
        return 0;
    });
}
int refh_alm_reduce_length(void* a, double fac) {
    return guard([&] {
        static_cast<RefALM*>(a)->alm->reduceLength(fac);
        return 0;
    });
}
// gsALMBase::isBifurcation / computeSingularPoint / switchBranch (gsALMBase.hpp:421-512, 628-852)
int refh_alm_is_bifurcation(void* a, int jacobian) {
    return guard([&] { return static_cast<RefALM*>(a)->alm->isBifurcation(jacobian != 0) ? 1 : 0; });
}
int refh_alm_compute_singular_point(void* a, const double* U, double L, int switch_branch, int jacobian,
                                    int test_point) {
    return guard([&] {
        RefALM* A = static_cast<RefALM*>(a);
        gsVector<real_t> u(A->P->n);
        std::memcpy(u.data(), U, sizeof(double) * A->P->n);
        return (int)A->alm->computeSingularPoint(u, L, switch_branch != 0, jacobian != 0, test_point != 0);
    });
}
int refh_alm_switch_branch(void* a) {
    return guard([&] {
        static_cast<RefALM*>(a)->alm->switchBranch();
        return 0;
    });
}
// out: [numIterations, indicator, stability, stabilityChange, getLength]
int refh_alm_info(void* a, double* out) {
    return guard([&] {
        gsALMBase<real_t>& A = *static_cast<RefALM*>(a)->alm;
        out[0] = A.numIterations();
        out[1] = A.indicator();
        out[2] = A.stability();
        out[3] = A.stabilityChange() ? 1 : 0;
        out[4] = A.getLength();
        return 0;
    });
}

// ---- gsStaticNewton ---------------------------------------------------------------------------
void* refh_newton_create(void* prob, const char* options) {
    RefProblem* P = static_cast<RefProblem*>(prob);
    RefNewton* out = nullptr;
    int st = guard([&] {
        typename gsStructuralAnalysisOps<real_t>::Jacobian_t J = [P](gsVector<real_t> const& x, gsSparseMatrix<real_t>& m) {
            return P->jacobian(x, m);
        };
        typename gsStructuralAnalysisOps<real_t>::Residual_t R = [P](gsVector<real_t> const& x, gsVector<real_t>& r) {
            r = gsVector<real_t>(P->n);
            return P->res(x.data(), r.data()) == 0;
        };
        std::unique_ptr<gsStaticNewton<real_t>> N(new gsStaticNewton<real_t>(P->KL, P->F, J, R));
        gsOptionList o;
        apply_options(o, options);
        N->setOptions(o);
        N->initialize();            // as the reference's drivers do (reset + getOptions)
        out = new RefNewton{P, std::move(N)};
        return 0;
    });
    return st == 0 ? out : nullptr;
}
void refh_newton_destroy(void* h) { delete static_cast<RefNewton*>(h); }
int refh_newton_solve(void* h) {
    return guard([&] { return (int)static_cast<RefNewton*>(h)->N->solve(); });
}
int refh_newton_solve_linear(void* h) {
    return guard([&] { return (int)static_cast<RefNewton*>(h)->N->solveLinear(); });
}
int refh_newton_set_displacement(void* h, const double* U) {
    return guard([&] {
        RefNewton* N = static_cast<RefNewton*>(h);
        gsVector<real_t> u(N->P->n);
        std::memcpy(u.data(), U, sizeof(double) * N->P->n);
        N->N->setDisplacement(u);
        return 0;
    });
}
int refh_newton_solution(void* h, double* U) {
    return guard([&] {
        RefNewton* N = static_cast<RefNewton*>(h);
        const gsVector<real_t>& u = N->N->solution();
        std::memcpy(U, u.data(), sizeof(double) * u.rows());
        return 0;
    });
}
int refh_newton_iterations(void* h) { return static_cast<RefNewton*>(h)->N->iterations(); }

// ---- dense eigenproblems: gsEigenProblemBase::compute / computePower --------------------------
// kind 0: gsModalSolver(A, B); kind 1: gsBucklingSolver(A, Bnl) with the pencil (A, Bnl - A).
// power != 0 runs computePower (one pair).  A, B: n x n column-major.  values: n (or 1),
// vectors: n x n (or n), column-major.  Returns the gsStatus, or -1.
int refh_eigen_dense(int kind, int n, const double* A, const double* B, const char* options, int power, double* values,
                     double* vectors) {
    return guard([&] {
        gsSparseMatrix<real_t> a(n, n), b(n, n);
        std::memcpy(a.data(), A, sizeof(double) * n * n);
        std::memcpy(b.data(), B, sizeof(double) * n * n);
        std::unique_ptr<gsEigenProblemBase<real_t>> E;
        if (kind == 0) E.reset(new gsModalSolver<real_t>(a, b));
        else E.reset(new gsBucklingSolver<real_t>(a, b));
        gsOptionList o;
        apply_options(o, options);
        E->setOptions(o);
        const gsStatus st = power ? E->computePower() : E->compute();
        const gsMatrix<real_t>& v = E->values();
        const gsMatrix<real_t>& V = E->vectors();
        std::memcpy(values, v.data(), sizeof(double) * v.size());
        std::memcpy(vectors, V.data(), sizeof(double) * V.size());
        return (int)st;
    });
}

// ---- gsAPALM over one of the arc-length methods above ------------------------------------------
// options: gsAPALM's (SubIntervals, MaxIt, ...); data_options: gsAPALMData's (MaxLevel,
// Tolerance), set on the empty data object the constructor takes
void* refh_apalm_create(void* alm, const char* options, const char* data_options) {
    RefAPALM* out = nullptr;
    int st = guard([&] {
        RefALM* A = static_cast<RefALM*>(alm);
        gsAPALMData<real_t, HarnessAPALM::solution_t> data;
        gsOptionList dopt;
        apply_options(dopt, data_options);
        data.options().update(dopt, gsOptionList::addIfUnknown);
        std::unique_ptr<HarnessAPALM> P(new HarnessAPALM(A->alm.get(), data));
        gsOptionList o;
        apply_options(o, options);
        P->options().update(o, gsOptionList::addIfUnknown);
        out = new RefAPALM{A, std::move(P)};
        return 0;
    });
    return st == 0 ? out : nullptr;
}
void refh_apalm_destroy(void* h) { delete static_cast<RefAPALM*>(h); }
int refh_apalm_initialize(void* h) {
    return guard([&] {
        static_cast<RefAPALM*>(h)->P->initialize();
        return 0;
    });
}
int refh_apalm_serial_solve(void* h, int nsteps) {
    return guard([&] {
        static_cast<RefAPALM*>(h)->P->serialSolve(nsteps);
        return 0;
    });
}
int refh_apalm_parallel_solve(void* h) {
    return guard([&] {
        static_cast<RefAPALM*>(h)->P->parallelSolve();
        return 0;
    });
}
int refh_apalm_solve(void* h, int nsteps) {
    return guard([&] {
        static_cast<RefAPALM*>(h)->P->solve(nsteps);
        return 0;
    });
}
int refh_apalm_branches(void* h) {
    return guard([&] { return (int)static_cast<RefAPALM*>(h)->P->branches(); });
}
// number of flat points of a branch (getFlatSolutions / getFlatTimes / getFlatLevels)
int refh_apalm_points(void* h, int branch) {
    return guard([&] { return (int)static_cast<RefAPALM*>(h)->P->getFlatTimes(branch).size(); });
}
int refh_apalm_point(void* h, int branch, int k, double* U, double* L, double* time, int* level) {
    return guard([&] {
        HarnessAPALM& P = *static_cast<RefAPALM*>(h)->P;
        const std::vector<HarnessAPALM::solution_t> sols = P.getFlatSolutions(branch);   // returned by value
        const auto& s = sols.at(k);
        std::memcpy(U, s.first.data(), sizeof(double) * s.first.rows());
        *L = s.second;
        *time = P.getFlatTimes(branch).at(k);
        *level = (int)P.getFlatLevels(branch).at(k);
        return 0;
    });
}

// ---- time integrators (gsDynamicBase and its subclasses) -------------------------------------
void* refh_dyn_create(int n, int64_t nnz, const int64_t* rowptr, const int32_t* cols, const char* method,
                      int nonlinear, refh_tmat_fn mass, refh_tmat_fn damping, refh_tmat_fn jac, refh_tvec_fn vec,
                      const char* options) {
    RefDyn* out = nullptr;
    int st = guard([&] {
        std::unique_ptr<RefDyn> D(new RefDyn());
        D->n = n;
        D->rowptr.assign(rowptr, rowptr + n + 1);
        D->cols.assign(cols, cols + nnz);
        D->mass = mass;
        D->damping = damping;
        D->jac = jac;
        D->vec = vec;
        const std::string m(method);
        const bool nl = nonlinear != 0;
        if (m == "Newmark") D->D.reset(make_dynamic<gsDynamicNewmark>(D.get(), nl));
        else if (m == "Bathe") D->D.reset(make_dynamic<gsDynamicBathe>(D.get(), nl));
        else if (m == "Wilson") D->D.reset(make_dynamic<gsDynamicWilson>(D.get(), nl));
        else if (m == "ExplicitEuler") D->D.reset(make_dynamic<gsDynamicExplicitEuler>(D.get(), nl));
        else if (m == "ImplicitEuler") D->D.reset(make_dynamic<gsDynamicImplicitEuler>(D.get(), nl));
        else if (m == "RK4") D->D.reset(make_dynamic<gsDynamicRK4>(D.get(), nl));
        else throw std::runtime_error("unknown integrator " + m);
        gsOptionList o;
        apply_options(o, options);
        D->D->setOptions(o);
        out = D.release();
        return 0;
    });
    return st == 0 ? out : nullptr;
}
void refh_dyn_destroy(void* h) { delete static_cast<RefDyn*>(h); }
int refh_dyn_set_state(void* h, const double* U, const double* V, const double* A) {
    return guard([&] {
        RefDyn* D = static_cast<RefDyn*>(h);
        gsVector<real_t> u(D->n), v(D->n), a(D->n);
        std::memcpy(u.data(), U, sizeof(double) * D->n);
        std::memcpy(v.data(), V, sizeof(double) * D->n);
        std::memcpy(a.data(), A, sizeof(double) * D->n);
        D->D->setU(u);
        D->D->setV(v);
        D->D->setA(a);
        return 0;
    });
}
// one step of size dt; returns the gsStatus, or -1
int refh_dyn_step(void* h, double dt) {
    return guard([&] { return (int)static_cast<RefDyn*>(h)->D->step(dt); });
}
// U, V, A (n each), time and the iteration count of the last step
int refh_dyn_state(void* h, double* U, double* V, double* A, double* info) {
    return guard([&] {
        gsDynamicBase<real_t>& D = *static_cast<RefDyn*>(h)->D;
        const gsVector<real_t>&u = D.solutionU(), &v = D.solutionV(), &a = D.solutionA();
        std::memcpy(U, u.data(), sizeof(double) * u.rows());
        std::memcpy(V, v.data(), sizeof(double) * v.rows());
        std::memcpy(A, a.data(), sizeof(double) * a.rows());
        info[0] = D.time();
        info[1] = D.numIterations();
        return 0;
    });
}

// gsBucklingSolver(K_L, F, Jacobian_t, scaling) (gsBucklingSolver.h:50-67, 127-149: u_L =
// K_L^-1 scaling F through SimplicialLDLT, B = K(u_L) - K_L) followed by computePower
// (gsEigenProblemBase.hpp:218-258).  value: 1, vector: n.  Returns the gsStatus, or -1.
int refh_buckling_power(void* prob, double scaling, const char* options, double* value, double* vector) {
    return guard([&] {
        RefProblem* P = static_cast<RefProblem*>(prob);
        typename gsStructuralAnalysisOps<real_t>::Jacobian_t J = [P](gsVector<real_t> const& x, gsSparseMatrix<real_t>& m) {
            return P->jacobian(x, m);
        };
        gsSparseMatrix<real_t> KL = P->KL;
        gsVector<real_t> F = P->F;
        gsBucklingSolver<real_t> B(KL, F, J, scaling);
        gsOptionList o;
        apply_options(o, options);
        B.options().update(o, gsOptionList::addIfUnknown);
        const gsStatus st = B.computePower();
        *value = B.values()(0, 0);
        std::memcpy(vector, B.vectors().data(), sizeof(double) * P->n);
        return (int)st;
    });
}

}  // extern "C"
