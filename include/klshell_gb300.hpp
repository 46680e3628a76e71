// klshell_gb300.hpp -- header-only C++ layer over the C-ABI of klshell_gb300.h, with the class and
// method names of the gsStructuralAnalysis solvers it replaces, for C++ drivers written against
// the reference:
//
//   klsa::Problem        gsThinShellAssembler + the Jacobian_t / Residual_t / ALResidual_t
//                        callbacks (gsStructuralAnalysisTools/gsStructuralAnalysisTypes.h:58-93)
//   klsa::StaticNewton   gsStaticNewton (gsStaticSolvers/gsStaticNewton.hpp)
//   klsa::ALM            gsALMCrisfield / gsALMRiks / gsALMLoadControl / gsALMConsistentCrisfield
//                        (gsALMSolvers/gsALMBase.h), chosen by name
//   klsa::APALM          gsAPALM (gsALMSolvers/gsAPALM.h)
//   klsa::Dynamic        gsDynamicNewmark / Bathe / Wilson / ExplicitEuler / ImplicitEuler / RK4
//                        (gsDynamicSolvers/gsDynamicBase.h)
//   klsa::buckling / klsa::modal   gsBucklingSolver / gsModalSolver
//
// Vectors are std::vector<double> in the reference's free-dof order.  Solver calls return the
// gsStatus code (0 Success, 1 NotConverged, 2 AssemblyError, 3 SolverError, 4 NotStarted,
// 5 OtherError) as the reference's solve()/step() do; negative ABI codes (invalid argument,
// CUDA error, unsupported) throw klsa::Error with the library's message.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "klshell_gb300.h"

namespace klsa {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

// negative codes are ABI errors; 0..5 are returned as gsStatus
inline int check(int code) {
    if (code < 0) {
        const char* m = klsa_last_error();
        throw Error(code, std::string("klsa status ") + std::to_string(code) + ": " + (m ? m : ""));
    }
    return code;
}

// gsOptionList-like key/value set handed to the solvers
class Options {
public:
    Options() : h_(klsa_options_create()) {
        if (!h_) throw Error(KLSA_OTHER_ERROR, "klsa_options_create failed");
    }
    ~Options() { klsa_options_destroy(h_); }
    Options(const Options&) = delete;
    Options& operator=(const Options&) = delete;
    Options& setReal(const std::string& k, double v) { check(klsa_options_set_real(h_, k.c_str(), v)); return *this; }
    Options& setInt(const std::string& k, int64_t v) { check(klsa_options_set_int(h_, k.c_str(), v)); return *this; }
    Options& setSwitch(const std::string& k, bool v) { return setInt(k, v ? 1 : 0); }
    Options& setString(const std::string& k, const std::string& v) {
        check(klsa_options_set_string(h_, k.c_str(), v.c_str()));
        return *this;
    }
    const klsa_options* get() const { return h_; }

private:
    klsa_options* h_;
};

// One patch on the device; its member functions are the reference's callbacks
class Problem {
public:
    explicit Problem(const klsa_patch_desc& d) { check(klsa_problem_create(&d, &h_)); }
    ~Problem() { if (h_) klsa_problem_destroy(h_); }
    Problem(const Problem&) = delete;
    Problem& operator=(const Problem&) = delete;
    klsa_problem* get() const { return h_; }
    int64_t numDofs() const { return klsa_problem_ndof(h_); }
    int64_t nonZeros() const { return klsa_problem_nnz(h_); }

    // Force_t
    std::vector<double> force() const {
        std::vector<double> F(numDofs());
        check(klsa_force(h_, F.data()));
        return F;
    }
    // Residual_t: R = Fext - Fint(x)
    bool residual(const std::vector<double>& x, std::vector<double>& R) const {
        R.resize(numDofs());
        return klsa_residual(h_, x.data(), R.data()) == KLSA_SUCCESS;
    }
    // ALResidual_t: R = Fint(x) - lambda F
    bool alResidual(const std::vector<double>& x, double lambda, std::vector<double>& R) const {
        R.resize(numDofs());
        return klsa_al_residual(h_, x.data(), lambda, R.data()) == KLSA_SUCCESS;
    }
    // Jacobian_t as CSR (rows sorted); fp64 = false: FP32 element integration
    struct CSR {
        std::vector<int64_t> rowptr;
        std::vector<int32_t> cols;
        std::vector<double> vals;
    };
    bool jacobian(const std::vector<double>& x, CSR& K, bool fp64 = true) const {
        K.rowptr.resize(numDofs() + 1);
        K.cols.resize(nonZeros());
        K.vals.resize(nonZeros());
        return klsa_jacobian_csr(h_, x.data(), fp64 ? 1 : 0, K.rowptr.data(), K.cols.data(), K.vals.data()) ==
               KLSA_SUCCESS;
    }
    // Mass_t
    bool mass(CSR& M) const {
        M.rowptr.resize(numDofs() + 1);
        M.cols.resize(nonZeros());
        M.vals.resize(nonZeros());
        return klsa_mass_csr(h_, M.rowptr.data(), M.cols.data(), M.vals.data()) == KLSA_SUCCESS;
    }

private:
    klsa_problem* h_ = nullptr;
};

// gsStaticNewton
class StaticNewton {
public:
    StaticNewton(Problem& P, const Options& o) : P_(P) { check(klsa_static_create(P.get(), o.get(), &h_)); }
    ~StaticNewton() { if (h_) klsa_static_destroy(h_); }
    StaticNewton(const StaticNewton&) = delete;
    StaticNewton& operator=(const StaticNewton&) = delete;
    int solve() { return check(klsa_static_solve(h_)); }
    int solveLinear() { return check(klsa_static_solve_linear(h_)); }
    void setLoad(double lambda) { check(klsa_static_set_load_factor(h_, lambda)); }
    void setDisplacement(const std::vector<double>& U) { check(klsa_static_set_displacement(h_, U.data())); }
    std::vector<double> solution() const {
        std::vector<double> U(P_.numDofs());
        check(klsa_static_solution(h_, U.data()));
        return U;
    }
    int numIterations() const { return klsa_static_iterations(h_); }

private:
    Problem& P_;
    klsa_static* h_ = nullptr;
};

// gsALMBase and subclasses: method "Crisfield", "Riks", "LoadControl", "ConsistentCrisfield"
class ALM {
public:
    ALM(Problem& P, const std::string& method, const Options& o) : P_(P) {
        check(klsa_alm_create(P.get(), method.c_str(), o.get(), &h_));
    }
    ~ALM() { if (h_) klsa_alm_destroy(h_); }
    ALM(const ALM&) = delete;
    ALM& operator=(const ALM&) = delete;
    klsa_alm* get() const { return h_; }
    int numDofs() const { return (int)P_.numDofs(); }
    void initialize(bool stability = true) { check(klsa_alm_initialize(h_, stability ? 1 : 0)); }
    int step() { return check(klsa_alm_step(h_)); }
    void setLength(double l) { check(klsa_alm_set_length(h_, l)); }
    double getLength() const { return klsa_alm_get_length(h_); }
    double reduceLength(double fac = 0.5) {
        check(klsa_alm_reduce_length(h_, fac));
        return getLength();
    }
    void setSolution(const std::vector<double>& U, double L) { check(klsa_alm_set_solution(h_, U.data(), L)); }
    void setSolutionStep(const std::vector<double>& DU, double DL) {
        check(klsa_alm_set_solution_step(h_, DU.data(), DL));
    }
    void setPrevious(const std::vector<double>& U, double L) { check(klsa_alm_set_previous(h_, U.data(), L)); }
    void setInitialGuess(const std::vector<double>& U, double L) {
        check(klsa_alm_set_initial_guess(h_, U.data(), L));
    }
    double distance(const std::vector<double>& DU, double DL) const {
        double d = 0.0;
        check(klsa_alm_distance(h_, DU.data(), DL, &d));
        return d;
    }
    std::vector<double> solutionU() const {
        std::vector<double> U(numDofs());
        double L = 0.0;
        check(klsa_alm_solution(h_, U.data(), &L));
        return U;
    }
    double solutionL() const {
        double L = 0.0;
        check(klsa_alm_solution(h_, nullptr, &L));
        return L;
    }
    std::vector<double> solutionV() const {
        std::vector<double> V(numDofs());
        check(klsa_alm_solution_v(h_, V.data()));
        return V;
    }
    int computeStability(bool jacobian = true, double shift = -1e2) {
        return check(klsa_alm_compute_stability(h_, jacobian ? 1 : 0, shift));
    }
    double indicator() const {
        double ind = 0.0;
        check(klsa_alm_stability(h_, &ind, nullptr, nullptr, nullptr));
        return ind;
    }
    int stability() const {
        int s = 0;
        check(klsa_alm_stability(h_, nullptr, &s, nullptr, nullptr));
        return s;
    }
    bool stabilityChange() const {
        int c = 0;
        check(klsa_alm_stability(h_, nullptr, nullptr, &c, nullptr));
        return c != 0;
    }
    bool isBifurcation(bool jacobian = false) { return check(klsa_alm_is_bifurcation(h_, jacobian ? 1 : 0)) == 1; }
    int computeSingularPoint(const std::vector<double>& U, double L, bool switchBranch = false, bool jacobian = false,
                             bool testPoint = true) {
        return check(klsa_alm_compute_singular_point(h_, U.data(), L, switchBranch, jacobian, testPoint));
    }
    void switchBranch() { check(klsa_alm_switch_branch(h_)); }

private:
    Problem& P_;
    klsa_alm* h_ = nullptr;
};

// gsAPALM over a Crisfield or Riks object
class APALM {
public:
    APALM(ALM& alm, const Options& o) : alm_(alm) { check(klsa_apalm_create(alm.get(), o.get(), &h_)); }
    ~APALM() { if (h_) klsa_apalm_destroy(h_); }
    APALM(const APALM&) = delete;
    APALM& operator=(const APALM&) = delete;
    void initialize() { check(klsa_apalm_initialize(h_)); }
    void serialSolve(int nsteps = 10) { check(klsa_apalm_serial_solve(h_, nsteps)); }
    void parallelSolve() { check(klsa_apalm_parallel_solve(h_)); }
    void solve(int nsteps = 10) { check(klsa_apalm_solve(h_, nsteps)); }
    int nBranches() const { return check(klsa_apalm_branches(h_)); }
    std::vector<std::pair<std::vector<double>, double>> getFlatSolutions(int branch = 0) const {
        const int n = check(klsa_apalm_solutions(h_, branch));
        std::vector<std::pair<std::vector<double>, double>> out(n);
        for (int k = 0; k < n; ++k) {
            out[k].first.resize(alm_.numDofs());
            check(klsa_apalm_solution(h_, branch, k, out[k].first.data(), &out[k].second, nullptr, nullptr));
        }
        return out;
    }
    std::vector<double> getFlatTimes(int branch = 0) const {
        const int n = check(klsa_apalm_solutions(h_, branch));
        std::vector<double> t(n);
        for (int k = 0; k < n; ++k) check(klsa_apalm_solution(h_, branch, k, nullptr, nullptr, &t[k], nullptr));
        return t;
    }
    std::vector<int> getFlatLevels(int branch = 0) const {
        const int n = check(klsa_apalm_solutions(h_, branch));
        std::vector<int> lv(n);
        for (int k = 0; k < n; ++k) check(klsa_apalm_solution(h_, branch, k, nullptr, nullptr, nullptr, &lv[k]));
        return lv;
    }

private:
    ALM& alm_;
    klsa_apalm* h_ = nullptr;
};

// gsDynamicBase and the integrators: "Newmark", "Bathe", "Wilson", "ExplicitEuler",
// "ImplicitEuler", "RK4"; nonlinear = the _NL template flag
class Dynamic {
public:
    Dynamic(Problem& P, const std::string& method, bool nonlinear, const Options& o) : P_(P) {
        check(klsa_dynamic_create(P.get(), method.c_str(), nonlinear ? 1 : 0, o.get(), &h_));
    }
    ~Dynamic() { if (h_) klsa_dynamic_destroy(h_); }
    Dynamic(const Dynamic&) = delete;
    Dynamic& operator=(const Dynamic&) = delete;
    void setLoadTable(const std::vector<double>& t, const std::vector<double>& f) {
        if (t.size() != f.size()) throw Error(KLSA_INVALID_ARGUMENT, "load table sizes differ");
        check(klsa_dynamic_set_load_table(h_, t.data(), f.data(), (int)t.size()));
    }
    void setU(const std::vector<double>& U) { check(klsa_dynamic_set_state(h_, U.data(), nullptr, nullptr)); }
    void setV(const std::vector<double>& V) { check(klsa_dynamic_set_state(h_, nullptr, V.data(), nullptr)); }
    void setA(const std::vector<double>& A) { check(klsa_dynamic_set_state(h_, nullptr, nullptr, A.data())); }
    std::vector<double> solutionU() const { return get(0); }
    std::vector<double> solutionV() const { return get(1); }
    std::vector<double> solutionA() const { return get(2); }
    int step(double dt = 0.0) { return check(klsa_dynamic_step(h_, dt)); }   // dt <= 0: option "DT"
    double time() const { return klsa_dynamic_time(h_); }
    void setTime(double t) { check(klsa_dynamic_set_time(h_, t)); }

private:
    std::vector<double> get(int which) const {
        std::vector<double> x(P_.numDofs());
        double* p[3] = {nullptr, nullptr, nullptr};
        p[which] = x.data();
        check(klsa_dynamic_state(h_, p[0], p[1], p[2]));
        return x;
    }
    Problem& P_;
    klsa_dynamic* h_ = nullptr;
};

// gsBucklingSolver / gsModalSolver: nev eigenpairs nearest shift (values; vectors nev x ndof)
inline int buckling(Problem& P, const Options& o, int nev, double shift, double scaling, std::vector<double>& values,
                    std::vector<double>* vectors = nullptr) {
    values.resize(nev);
    if (vectors) vectors->resize((size_t)nev * P.numDofs());
    return check(klsa_buckling(P.get(), o.get(), nev, shift, scaling, values.data(),
                               vectors ? vectors->data() : nullptr));
}
inline int modal(Problem& P, const Options& o, int nev, double shift, std::vector<double>& values,
                 std::vector<double>* vectors = nullptr) {
    values.resize(nev);
    if (vectors) vectors->resize((size_t)nev * P.numDofs());
    return check(klsa_modal(P.get(), o.get(), nev, shift, values.data(), vectors ? vectors->data() : nullptr));
}

}  // namespace klsa
