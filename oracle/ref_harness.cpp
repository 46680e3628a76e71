// CPU oracle built from the reference's OWN solver headers (test infrastructure only).
//
// gsStaticNewton, gsALMCrisfield, gsALMRiks, gsALMLoadControl, gsALMConsistentCrisfield,
// gsModalSolver and gsBucklingSolver are compiled unchanged from the reference tree
// (src/gsStaticSolvers, src/gsALMSolvers, src/gsEigenSolvers) against the test-only stand-in of
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
#include <gsStructuralAnalysis/src/gsALMSolvers/gsALMCrisfield.h>
#include <gsStructuralAnalysis/src/gsALMSolvers/gsALMLoadControl.h>
#include <gsStructuralAnalysis/src/gsALMSolvers/gsALMRiks.h>
#include <gsStructuralAnalysis/src/gsEigenSolvers/gsBucklingSolver.h>
#include <gsStructuralAnalysis/src/gsEigenSolvers/gsModalSolver.h>
#include <gsStructuralAnalysis/src/gsStaticSolvers/gsStaticNewton.h>

using namespace gismo;

extern "C" {
// x: free-dof vector; vals: the Jacobian's values in the problem's fixed CSR pattern
typedef int (*refh_jac_fn)(const double* x, double* vals);
// Fint(x) - lambda F  (ALResidual_t)
typedef int (*refh_alres_fn)(const double* x, double lambda, double* R);
// F - Fint(x)  (Residual_t)
typedef int (*refh_res_fn)(const double* x, double* R);
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

}  // extern "C"
