// capi.cu -- extern "C" entry points (include/klshell_gb300.h).  No exception crosses the ABI.
#include <cstring>
#include <exception>
#include <memory>
#include <string>

#include "../../include/klshell_gb300.h"
#include "apalm.h"
#include "batch.h"
#include "dynamics.h"
#include "eigen.h"
#include "linalg.h"
#include "mlp.h"
#include "predictor.h"
#include "problem.h"
#include "solvers.h"

using namespace klsa;

struct klsa_problem {
    std::unique_ptr<Problem> P;
    DevBuf<double> x, r, f;   // staging (internal order)
    cudaEvent_t ev[16] = {};
    ~klsa_problem() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }
};
struct klsa_options {
    Options o;
};
struct klsa_solver {
    klsa_problem* prob;
    std::unique_ptr<LinearSolver> S;
    DevBuf<double> b, x;
};
struct klsa_static {
    klsa_problem* prob;
    std::unique_ptr<StaticNewtonGPU> N;
};
struct klsa_alm {
    klsa_problem* prob;
    std::unique_ptr<ALMGPU> A;
    DevBuf<double> v;
};
struct klsa_apalm {
    klsa_alm* alm;
    std::unique_ptr<APALM> A;
};
struct klsa_dynamic {
    klsa_problem* prob;
    std::unique_ptr<DynamicGPU> D;
};
struct klsa_mlp {
    std::unique_ptr<MLP> net;
};
struct klsa_predictor {
    klsa_problem* prob;
    std::unique_ptr<LearnedPredictor> pred;
    DevBuf<double> ug, u;
};

struct klsa_batch {
    std::unique_ptr<BatchedProblem> B;
    cudaEvent_t ev[16] = {};
    ~klsa_batch() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }
};
struct klsa_batch_newton {
    klsa_batch* b;
    std::unique_ptr<BatchedNewton> N;
};

namespace {

thread_local std::string g_err;

template <class F>
int guarded(F&& f) {
    try {
        return f();
    } catch (const CudaError& e) {
        g_err = e.what();
        return KLSA_CUDA_ERROR;
    } catch (const std::invalid_argument& e) {
        g_err = e.what();
        return KLSA_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        g_err = e.what();
        return KLSA_OTHER_ERROR;
    } catch (...) {
        g_err = "unknown error";
        return KLSA_OTHER_ERROR;
    }
}

void ensure(DevBuf<double>& b, size_t n) {
    if (b.size() < n) b.alloc(n);
}

}  // namespace

void klsa_set_error(const std::string& msg) { g_err = msg; }
klsa::Problem* klsa_problem_impl(klsa_problem* prob) { return prob->P.get(); }

extern "C" {

const char* klsa_last_error(void) { return g_err.c_str(); }
uint64_t klsa_launch_count(void) { return (uint64_t)g_launch_count; }

int klsa_problem_create(const klsa_patch_desc* desc, klsa_problem** out) {
    if (!desc || !out) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        auto h = new klsa_problem();
        try {
            h->P.reset(new Problem(*desc));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
        return KLSA_SUCCESS;
    });
}

int klsa_problem_destroy(klsa_problem* prob) {
    return guarded([&] {
        delete prob;
        return KLSA_SUCCESS;
    });
}

int64_t klsa_problem_ndof(const klsa_problem* prob) { return prob ? prob->P->nfree : -1; }
int64_t klsa_problem_nnz(const klsa_problem* prob) { return prob ? prob->P->nnz : -1; }

int klsa_force(klsa_problem* prob, double* F) {
    if (!prob || !F) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        prob->P->download_pub(prob->P->d_F.get(), F);
        return KLSA_SUCCESS;
    });
}

static int residual_impl(klsa_problem* prob, const double* x, double lambda, bool al, double* R) {
    if (!prob || !x || !R) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *prob->P;
        ensure(prob->x, P.nfree); ensure(prob->r, P.nfree); ensure(prob->f, P.nfree);
        P.upload_pub(x, prob->x.get());
        cudaEvent_t ev = g_timer.begin(P.stream);
        P.set_displacement(prob->x.get());
        P.internal_force(prob->f.get());
        if (al) vec::lincomb(1.0, prob->f.get(), -lambda, P.d_F.get(), prob->r.get(), P.nfree, P.stream);
        else vec::lincomb(1.0, P.d_F.get(), -1.0, prob->f.get(), prob->r.get(), P.nfree, P.stream);
        g_timer.end(P.stream, 3, ev);
        P.download_pub(prob->r.get(), R);
        return KLSA_SUCCESS;
    });
}

int klsa_residual(klsa_problem* prob, const double* x, double* R) { return residual_impl(prob, x, 0.0, false, R); }
int klsa_al_residual(klsa_problem* prob, const double* x, double lambda, double* R) {
    return residual_impl(prob, x, lambda, true, R);
}

int klsa_jacobian_csr(klsa_problem* prob, const double* x, int precision, int64_t* rowptr, int32_t* cols,
                      double* vals) {
    if (!prob || !x || !rowptr || !cols || !vals) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *prob->P;
        ensure(prob->x, P.nfree);
        P.upload_pub(x, prob->x.get());
        P.set_displacement(prob->x.get());
        if (precision) P.tangent_f64(); else P.tangent_f32();
        P.csr_to_host_pub(precision != 0, rowptr, cols, vals);
        return KLSA_SUCCESS;
    });
}

int klsa_djacobian_csr(klsa_problem* prob, const double* x, const double* dx, int precision, int64_t* rowptr,
                       int32_t* cols, double* vals) {
    // The tangent at x.  The increment dx is part of the signature the solvers call
    // (gsALMBase.hpp:214-223, gsStaticNewton.hpp:205-212) and is not used by this material: the
    // reference itself builds its dJacobian from a Jacobian this way (gsALMBase.h:57-60,
    // gsStaticNewton.h:79-82).
    if (!dx) return KLSA_INVALID_ARGUMENT;
    return klsa_jacobian_csr(prob, x, precision, rowptr, cols, vals);
}

int klsa_mass_csr(klsa_problem* prob, int64_t* rowptr, int32_t* cols, double* vals) {
    if (!prob || !rowptr || !cols || !vals) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        prob->P->mass_f64();
        prob->P->csr_to_host_pub(true, rowptr, cols, vals);
        return KLSA_SUCCESS;
    });
}

klsa_options* klsa_options_create(void) { return new klsa_options(); }
void klsa_options_destroy(klsa_options* opt) { delete opt; }
int klsa_options_set_real(klsa_options* opt, const char* key, double value) {
    if (!opt || !key) return KLSA_INVALID_ARGUMENT;
    opt->o.reals[key] = value;
    opt->o.ints.erase(key);
    return KLSA_SUCCESS;
}
int klsa_options_set_int(klsa_options* opt, const char* key, int64_t value) {
    if (!opt || !key) return KLSA_INVALID_ARGUMENT;
    opt->o.ints[key] = value;
    opt->o.reals.erase(key);
    return KLSA_SUCCESS;
}
int klsa_options_set_string(klsa_options* opt, const char* key, const char* value) {
    if (!opt || !key || !value) return KLSA_INVALID_ARGUMENT;
    opt->o.strs[key] = value;
    return KLSA_SUCCESS;
}

int klsa_solver_create(klsa_problem* prob, const char* name, const klsa_options* opt, klsa_solver** out) {
    if (!prob || !name || !out) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Options o = opt ? opt->o : Options();
        auto s = make_linear_solver(*prob->P, name, (int)o.integer("Refinement", 0), o.real("RefineTol", 1e-12),
                                    (int)o.integer("CGMaxIterations", 0), o.real("CGTolerance", 1e-10),
                                    (int)o.integer("FrontPrecision", 32));
        if (!s) {
            g_err = std::string("unknown solver name ") + name;
            return KLSA_INVALID_ARGUMENT;
        }
        auto h = new klsa_solver();
        h->prob = prob;
        h->S = std::move(s);
        *out = h;
        return KLSA_SUCCESS;
    });
}

int klsa_solver_destroy(klsa_solver* s) {
    return guarded([&] {
        delete s;
        return KLSA_SUCCESS;
    });
}

int klsa_solver_compute_jacobian(klsa_solver* s, const double* x) {
    if (!s || !x) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *s->prob->P;
        ensure(s->x, P.nfree);
        P.upload_pub(x, s->x.get());
        P.set_displacement(s->x.get());
        return s->S->compute_tangent();
    });
}

int klsa_solver_compute_linear(klsa_solver* s) {
    if (!s) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *s->prob->P;
        ensure(s->x, P.nfree);
        s->x.zero(P.stream);
        P.set_displacement(s->x.get());
        return s->S->compute_tangent();
    });
}

int klsa_solver_solve(klsa_solver* s, const double* b, double* x, int nrhs) {
    if (!s || !b || !x || nrhs < 1 || nrhs > MF_MAX_RHS) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *s->prob->P;
        ensure(s->b, (size_t)P.nfree * nrhs);
        ensure(s->x, (size_t)P.nfree * nrhs);
        P.upload_pub(b, s->b.get(), nrhs);
        int st = s->S->solve(s->b.get(), s->x.get(), nrhs);
        if (st != KLSA_SUCCESS) return st;
        P.download_pub(s->x.get(), x, nrhs);
        return KLSA_SUCCESS;
    });
}

int klsa_solver_iterations(klsa_solver* s) { return s ? s->S->last_iterations() : KLSA_INVALID_ARGUMENT; }

int klsa_solver_stability(klsa_solver* s, double* min_d, int64_t* negatives) {
    if (!s || !min_d || !negatives) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        if (!s->S->has_ldlt()) {
            g_err = "determinant stability needs the LDL^T solver";
            return KLSA_SOLVER_ERROR;
        }
        s->S->stability(min_d, negatives);
        return KLSA_SUCCESS;
    });
}

// ---- static Newton ------------------------------------------------------------------------
int klsa_static_create(klsa_problem* prob, const klsa_options* opt, klsa_static** out) {
    if (!prob || !out) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        auto h = new klsa_static();
        h->prob = prob;
        try {
            h->N.reset(new StaticNewtonGPU(*prob->P, opt ? opt->o : Options()));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
        return KLSA_SUCCESS;
    });
}
int klsa_static_destroy(klsa_static* s) {
    return guarded([&] {
        delete s;
        return KLSA_SUCCESS;
    });
}
int klsa_static_solve(klsa_static* s) {
    if (!s) return KLSA_INVALID_ARGUMENT;
    return guarded([&] { return s->N->solve(); });
}
int klsa_static_solve_linear(klsa_static* s) {
    if (!s) return KLSA_INVALID_ARGUMENT;
    return guarded([&] { return s->N->solve_linear(); });
}
int klsa_static_set_load_factor(klsa_static* s, double lambda) {
    if (!s) return KLSA_INVALID_ARGUMENT;
    s->N->set_load(lambda);
    return KLSA_SUCCESS;
}
int klsa_static_set_displacement(klsa_static* s, const double* U) {
    if (!s || !U) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *s->prob->P;
        ensure(s->prob->x, P.nfree);
        P.upload_pub(U, s->prob->x.get());
        s->N->set_displacement(s->prob->x.get());
        return KLSA_SUCCESS;
    });
}
int klsa_static_solution(klsa_static* s, double* U) {
    if (!s || !U) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        s->prob->P->download_pub(s->N->solution(), U);
        return KLSA_SUCCESS;
    });
}
int klsa_static_iterations(klsa_static* s) { return s ? s->N->iterations() : -1; }

// ---- arc-length -----------------------------------------------------------------------------
int klsa_alm_create(klsa_problem* prob, const char* method, const klsa_options* opt, klsa_alm** out) {
    if (!prob || !method || !out) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        ALMGPU::Method m;
        std::string s(method);
        if (s == "Crisfield") m = ALMGPU::Crisfield;
        else if (s == "Riks") m = ALMGPU::Riks;
        else if (s == "LoadControl") m = ALMGPU::LoadControl;
        else if (s == "ConsistentCrisfield") m = ALMGPU::ConsistentCrisfield;
        else {
            g_err = "unknown arc-length method " + s;
            return KLSA_INVALID_ARGUMENT;
        }
        auto h = new klsa_alm();
        h->prob = prob;
        try {
            h->A.reset(new ALMGPU(*prob->P, m, opt ? opt->o : Options()));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
        return KLSA_SUCCESS;
    });
}
int klsa_alm_destroy(klsa_alm* a) {
    return guarded([&] {
        delete a;
        return KLSA_SUCCESS;
    });
}
int klsa_alm_initialize(klsa_alm* a, int stability) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        a->A->initialize(false);
        return stability ? a->A->compute_stability(true, -1e2) : KLSA_SUCCESS;
    });
}
int klsa_alm_compute_stability(klsa_alm* a, int jacobian, double shift) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    return guarded([&] { return a->A->compute_stability(jacobian != 0, shift); });
}
int klsa_alm_stability(klsa_alm* a, double* indicator, int* stability, int* change, int64_t* negatives) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    if (indicator) *indicator = a->A->indicator();
    if (stability) *stability = a->A->stability();
    if (change) *change = a->A->stability_change() ? 1 : 0;
    if (negatives) *negatives = a->A->negatives();
    return KLSA_SUCCESS;
}
int klsa_alm_step(klsa_alm* a) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    return guarded([&] { return a->A->step(); });
}
int klsa_alm_set_length(klsa_alm* a, double length) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    a->A->set_length(length);
    return KLSA_SUCCESS;
}
int klsa_alm_reduce_length(klsa_alm* a, double factor) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    a->A->reduce_length(factor);
    return KLSA_SUCCESS;
}
double klsa_alm_get_length(klsa_alm* a) { return a ? a->A->length() : -1.0; }
int klsa_alm_set_solution(klsa_alm* a, const double* U, double L) {
    if (!a || !U) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *a->prob->P;
        ensure(a->v, P.nfree);
        P.upload_pub(U, a->v.get());
        a->A->set_solution(a->v.get(), L);
        return KLSA_SUCCESS;
    });
}
int klsa_alm_set_previous(klsa_alm* a, const double* Uprev, double Lprev) {
    if (!a || !Uprev) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *a->prob->P;
        ensure(a->prob->x, P.nfree);
        P.upload_pub(Uprev, a->prob->x.get());
        a->A->set_previous(a->prob->x.get(), Lprev);
        KL_CUDA(cudaStreamSynchronize(P.stream));
        return KLSA_SUCCESS;
    });
}
int klsa_alm_distance(klsa_alm* a, const double* DU, double DL, double* out) {
    if (!a || !DU || !out) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *a->prob->P;
        ensure(a->prob->x, P.nfree);
        P.upload_pub(DU, a->prob->x.get());
        *out = a->A->distance(a->prob->x.get(), DL);
        return KLSA_SUCCESS;
    });
}
int klsa_alm_set_solution_step(klsa_alm* a, const double* DU, double DL) {
    if (!a || !DU) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *a->prob->P;
        ensure(a->v, P.nfree);
        P.upload_pub(DU, a->v.get());
        a->A->set_solution_step(a->v.get(), DL);
        return KLSA_SUCCESS;
    });
}
int klsa_alm_set_initial_guess(klsa_alm* a, const double* U, double L) {
    if (!a || !U) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *a->prob->P;
        ensure(a->v, P.nfree);
        P.upload_pub(U, a->v.get());
        a->A->set_initial_guess(a->v.get(), L);
        return KLSA_SUCCESS;
    });
}
int klsa_alm_solution(klsa_alm* a, double* U, double* L) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        if (U) a->prob->P->download_pub(a->A->U(), U);
        if (L) *L = a->A->L();
        return KLSA_SUCCESS;
    });
}
int klsa_alm_is_bifurcation(klsa_alm* a, int jacobian) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    return guarded([&] { return a->A->is_bifurcation(jacobian != 0) ? 1 : 0; });
}
int klsa_alm_compute_singular_point(klsa_alm* a, const double* U, double L, int switch_branch, int jacobian,
                                    int test_point) {
    if (!a || !U) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *a->prob->P;
        ensure(a->v, P.nfree);
        P.upload_pub(U, a->v.get());
        return a->A->compute_singular_point(a->v.get(), L, switch_branch != 0, jacobian != 0, test_point != 0);
    });
}
int klsa_alm_switch_branch(klsa_alm* a) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        a->A->switch_branch();
        return KLSA_SUCCESS;
    });
}
int klsa_alm_solution_v(klsa_alm* a, double* V) {
    if (!a || !V) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        if (!a->A->V()) {
            g_err = "no singular-point vector computed";
            return KLSA_INVALID_ARGUMENT;
        }
        a->prob->P->download_pub(a->A->V(), V);
        return KLSA_SUCCESS;
    });
}
int klsa_alm_info(klsa_alm* a, double* out) {
    if (!a || !out) return KLSA_INVALID_ARGUMENT;
    out[0] = a->A->iterations();
    out[1] = a->A->residueF();
    out[2] = a->A->residueU();
    out[3] = a->A->phi();
    out[4] = a->A->converged() ? 1.0 : 0.0;
    out[5] = a->A->Lprev();
    out[6] = a->A->DLold();
    out[7] = a->A->n_jac;
    out[8] = a->A->n_res;
    out[9] = a->A->n_solve;
    return KLSA_SUCCESS;
}
int klsa_alm_history(klsa_alm* a, double* Uprev, double* Lprev, double* DUold, double* DLold) {
    if (!a) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        if (Uprev) a->prob->P->download_pub(a->A->Uprev(), Uprev);
        if (DUold) a->prob->P->download_pub(a->A->DUold(), DUold);
        if (Lprev) *Lprev = a->A->Lprev();
        if (DLold) *DLold = a->A->DLold();
        return KLSA_SUCCESS;
    });
}

// ---- measurement helpers ----------------------------------------------------------------------
int klsa_profile_enable(int on) {
    g_timer.collect();
    g_timer.enabled = on != 0;
    return KLSA_SUCCESS;
}
int klsa_profile_read(double* ms, uint64_t* counts) {
    return guarded([&] {
        g_timer.collect();
        for (int i = 0; i < PhaseTimer::NPH; ++i) {
            if (ms) ms[i] = g_timer.ms[i];
            if (counts) counts[i] = g_timer.count[i];
        }
        return KLSA_SUCCESS;
    });
}
int klsa_profile_reset(void) {
    return guarded([&] {
        g_timer.reset();
        return KLSA_SUCCESS;
    });
}
int klsa_event_record(klsa_problem* prob, int slot) {
    if (!prob || slot < 0 || slot >= 16) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        if (!prob->ev[slot]) KL_CUDA(cudaEventCreate(&prob->ev[slot]));
        KL_CUDA(cudaEventRecord(prob->ev[slot], prob->P->stream));
        return KLSA_SUCCESS;
    });
}
int klsa_event_elapsed(klsa_problem* prob, int slot_a, int slot_b, float* ms) {
    if (!prob || !ms || slot_a < 0 || slot_a >= 16 || slot_b < 0 || slot_b >= 16) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        if (!prob->ev[slot_a] || !prob->ev[slot_b]) return KLSA_INVALID_ARGUMENT;
        KL_CUDA(cudaEventSynchronize(prob->ev[slot_b]));
        KL_CUDA(cudaEventElapsedTime(ms, prob->ev[slot_a], prob->ev[slot_b]));
        return KLSA_SUCCESS;
    });
}
int klsa_problem_sync(klsa_problem* prob) {
    if (!prob) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        KL_CUDA(cudaStreamSynchronize(prob->P->stream));
        return KLSA_SUCCESS;
    });
}
int klsa_problem_stats(klsa_problem* prob, double* out) {
    if (!prob || !out) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *prob->P;
        Multifrontal& mf = P.solver();
        out[0] = P.nfree;
        out[1] = (double)P.nnz;
        out[2] = P.nel;
        out[3] = P.nqp;
        out[4] = (double)mf.front_bytes();
        out[5] = mf.flops();
        out[6] = P.flops_tangent();
        out[7] = (double)P.tree.nodes.size();
        for (int i = 0; i < 3; ++i) {
            out[8 + i] = mf.kernel_bytes[i];
            out[11 + i] = mf.kernel_flops[i];
            out[14 + i] = mf.kernel_launches[i];
        }
        out[17] = mf.solve_bytes;
        return KLSA_SUCCESS;
    });
}

// ---- learned predictor ------------------------------------------------------------------------
int klsa_mlp_create(int n_in, int n_h1, int n_h2, int n_out, uint64_t seed, klsa_mlp** out) {
    if (!out || n_in < 1 || n_h1 < 1 || n_h2 < 1 || n_out < 1) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        auto h = new klsa_mlp();
        try {
            h->net.reset(new MLP(n_in, n_h1, n_h2, n_out, seed));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
        return KLSA_SUCCESS;
    });
}
int klsa_mlp_destroy(klsa_mlp* net) {
    return guarded([&] {
        delete net;
        return KLSA_SUCCESS;
    });
}
int64_t klsa_mlp_num_params(const klsa_mlp* net) { return net ? net->net->nparams : -1; }
int klsa_mlp_get_params(klsa_mlp* net, float* params) {
    if (!net || !params) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        MLP& m = *net->net;
        KL_CUDA(cudaMemcpyAsync(params, m.params.get(), sizeof(float) * m.nparams, cudaMemcpyDeviceToHost, m.stream));
        KL_CUDA(cudaStreamSynchronize(m.stream));
        return KLSA_SUCCESS;
    });
}
int klsa_mlp_set_params(klsa_mlp* net, const float* params) {
    if (!net || !params) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        MLP& m = *net->net;
        KL_CUDA(cudaMemcpyAsync(m.params.get(), params, sizeof(float) * m.nparams, cudaMemcpyHostToDevice, m.stream));
        m.m.zero(m.stream);
        m.v.zero(m.stream);
        m.t_adam = 0;
        KL_CUDA(cudaStreamSynchronize(m.stream));
        return KLSA_SUCCESS;
    });
}
int klsa_mlp_forward(klsa_mlp* net, const float* X, int batch, float* Y) {
    if (!net || !X || !Y || batch < 1) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        MLP& m = *net->net;
        DevBuf<float> dX;
        dX.upload(X, (size_t)batch * m.in, m.stream);
        m.forward(dX.get(), batch);
        KL_CUDA(cudaMemcpyAsync(Y, m.Y.get(), sizeof(float) * batch * m.out, cudaMemcpyDeviceToHost, m.stream));
        KL_CUDA(cudaStreamSynchronize(m.stream));
        return KLSA_SUCCESS;
    });
}
int klsa_mlp_loss_grad(klsa_mlp* net, const float* X, const float* T, int batch, float* loss, float* grad) {
    if (!net || !X || !T || batch < 1) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        MLP& m = *net->net;
        DevBuf<float> dX, dT;
        dX.upload(X, (size_t)batch * m.in, m.stream);
        dT.upload(T, (size_t)batch * m.out, m.stream);
        float l = m.loss_grad(dX.get(), dT.get(), batch);
        if (loss) *loss = l;
        if (grad) {
            KL_CUDA(cudaMemcpyAsync(grad, m.grad.get(), sizeof(float) * m.nparams, cudaMemcpyDeviceToHost, m.stream));
            KL_CUDA(cudaStreamSynchronize(m.stream));
        }
        return KLSA_SUCCESS;
    });
}
int klsa_mlp_train(klsa_mlp* net, const float* X, const float* T, int nsamples, int epochs, int batch, float lr,
                   uint64_t seed, float* final_loss) {
    if (!net || !X || !T || nsamples < 1 || epochs < 0 || batch < 1) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        float l = net->net->train(X, T, nsamples, epochs, batch, lr, seed);
        if (final_loss) *final_loss = l;
        return KLSA_SUCCESS;
    });
}
int klsa_predictor_create(klsa_problem* prob, klsa_mlp* net, const double* modes, int nmodes, const double* in_mean,
                          const double* in_std, const double* out_mean, const double* out_std, klsa_predictor** out) {
    if (!prob || !out || nmodes < 0 || (nmodes > 0 && !modes)) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        auto h = new klsa_predictor();
        h->prob = prob;
        try {
            h->pred.reset(new LearnedPredictor(*prob->P, net ? net->net.get() : nullptr, modes, nmodes, in_mean, in_std,
                                               out_mean, out_std));
            h->ug.alloc(prob->P->nfree);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
        return KLSA_SUCCESS;
    });
}
int klsa_predictor_destroy(klsa_predictor* pr) {
    return guarded([&] {
        delete pr;
        return KLSA_SUCCESS;
    });
}
int klsa_predictor_reset(klsa_predictor* pr) {
    if (!pr) return KLSA_INVALID_ARGUMENT;
    pr->pred->reset();
    return KLSA_SUCCESS;
}
int klsa_predictor_push(klsa_predictor* pr, const double* U, double L) {
    if (!pr || !U) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *pr->prob->P;
        P.upload_pub(U, pr->ug.get());
        pr->pred->push(pr->ug.get(), L);
        return KLSA_SUCCESS;
    });
}
int klsa_predictor_guess(klsa_predictor* pr, double* U, double* L, int* available) {
    if (!pr || !U || !L) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *pr->prob->P;
        double Lg = 0.0;
        const bool ok = pr->pred->guess(pr->ug.get(), &Lg);
        if (available) *available = ok ? 1 : 0;
        if (ok) {
            P.download_pub(pr->ug.get(), U);
            *L = Lg;
        }
        return KLSA_SUCCESS;
    });
}
int klsa_alm_step_learned(klsa_alm* a, klsa_predictor* pr, int guess_max_iter, int* used_guess) {
    if (!a || !pr || pr->prob != a->prob) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        ALMGPU& A = *a->A;
        LearnedPredictor& L = *pr->pred;
        if (used_guess) *used_guess = 0;
        if (L.count == 0) L.push(A.U(), A.L());
        double Lg = 0.0;
        const double* Lcorr = nullptr;
        if (L.guess_deferred(pr->ug.get(), &Lg, &Lcorr)) {
            A.set_initial_guess_dev(pr->ug.get(), Lg, Lcorr);
            A.set_guess_place(true);
            int saved = A.max_iter();
            A.set_max_iter(guess_max_iter > 1 ? guess_max_iter : saved);
            int st = A.step();
            A.set_max_iter(saved);
            A.set_guess_place(false);
            if (st == KLSA_SUCCESS) {
                L.push(A.U(), A.L());
                if (used_guess) *used_guess = 1;
                return KLSA_SUCCESS;
            }
        }
        int st = A.step();   // plain tangent predictor (the state is unchanged by a failed attempt)
        if (st == KLSA_SUCCESS) L.push(A.U(), A.L());
        return st;
    });
}

// ---- eigen problems ---------------------------------------------------------------------------
int klsa_buckling(klsa_problem* prob, const klsa_options* opt, int nev, double shift, double scaling,
                  double* values, double* vectors) {
    if (!prob || !values || nev < 1) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        return buckling_gpu(*prob->P, opt ? opt->o : Options(), nev, shift, scaling, values, vectors);
    });
}

int klsa_modal(klsa_problem* prob, const klsa_options* opt, int nev, double shift, double* values, double* vectors) {
    if (!prob || !values || nev < 1) return KLSA_INVALID_ARGUMENT;
    return guarded([&] { return modal_gpu(*prob->P, opt ? opt->o : Options(), nev, shift, values, vectors); });
}

int klsa_eigen_dense(klsa_problem* prob, const klsa_options* opt, int kind, double scaling, double* values,
                     double* vectors) {
    if (!prob || !values || (kind != 0 && kind != 1)) return KLSA_INVALID_ARGUMENT;
    if (prob->P->nfree > 4096) {
        klsa_set_error("klsa_eigen_dense: the dense eigensolver holds n x n matrices; at most 4096 dofs (use "
                       "klsa_modal / klsa_buckling for sparse sizes)");
        return KLSA_INVALID_ARGUMENT;
    }
    return guarded([&] { return dense_gpu(*prob->P, opt ? opt->o : Options(), kind, scaling, values, vectors); });
}

int klsa_eigen_power(klsa_problem* prob, const klsa_options* opt, int kind, double scaling, double* value,
                     double* vector) {
    if (!prob || !value || (kind != 0 && kind != 1)) return KLSA_INVALID_ARGUMENT;
    return guarded([&] { return power_gpu(*prob->P, opt ? opt->o : Options(), kind, scaling, value, vector); });
}

// ---- adaptive parallel arc-length method -----------------------------------------------------
int klsa_apalm_create(klsa_alm* alm, const klsa_options* opt, klsa_apalm** out) {
    if (!alm || !out) return KLSA_INVALID_ARGUMENT;
    *out = nullptr;
    return guarded([&] {
        std::unique_ptr<klsa_apalm> h(new klsa_apalm);
        h->alm = alm;
        h->A.reset(new APALM(*alm->A, opt ? opt->o : Options()));
        *out = h.release();
        return KLSA_SUCCESS;
    });
}
int klsa_apalm_destroy(klsa_apalm* ap) {
    return guarded([&] {
        delete ap;
        return KLSA_SUCCESS;
    });
}
int klsa_apalm_add_worker(klsa_apalm* ap, klsa_alm* worker) {
    if (!ap || !worker) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        ap->A->add_worker(*worker->A, *worker->prob->P);
        return KLSA_SUCCESS;
    });
}
int klsa_apalm_initialize(klsa_apalm* ap) {
    if (!ap) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        ap->A->initialize();
        return KLSA_SUCCESS;
    });
}
int klsa_apalm_add_start(klsa_apalm* ap, const double* U, double L, double dL) {
    if (!ap || !U) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *ap->alm->prob->P;
        ensure(ap->alm->prob->x, P.nfree);
        P.upload_pub(U, ap->alm->prob->x.get());
        ap->A->add_start(ap->alm->prob->x.get(), L, dL);
        KL_CUDA(cudaStreamSynchronize(P.stream));
        return KLSA_SUCCESS;
    });
}
int klsa_apalm_serial_solve(klsa_apalm* ap, int nsteps) {
    if (!ap) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        ap->A->serial_solve(nsteps);
        return KLSA_SUCCESS;
    });
}
int klsa_apalm_parallel_solve(klsa_apalm* ap) {
    if (!ap) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        ap->A->parallel_solve();
        return KLSA_SUCCESS;
    });
}
int klsa_apalm_solve(klsa_apalm* ap, int nsteps) {
    if (!ap) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        ap->A->solve(nsteps);
        return KLSA_SUCCESS;
    });
}
int klsa_apalm_branches(klsa_apalm* ap) { return ap ? ap->A->branches() : KLSA_INVALID_ARGUMENT; }
int klsa_apalm_solutions(klsa_apalm* ap, int branch) {
    if (!ap || branch < 0 || branch >= ap->A->branches()) return KLSA_INVALID_ARGUMENT;
    return ap->A->solutions(branch);
}
int klsa_apalm_solution(klsa_apalm* ap, int branch, int k, double* U, double* L, double* time, int* level) {
    if (!ap || branch < 0 || branch >= ap->A->branches() || k < 0 || k >= ap->A->solutions(branch))
        return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        const APSolution& s = ap->A->solution(branch, k);
        if (U) ap->alm->prob->P->download_pub(s.U->get(), U);
        if (L) *L = s.L;
        if (time) *time = ap->A->time(branch, k);
        if (level) *level = ap->A->level(branch, k);
        return KLSA_SUCCESS;
    });
}

// ---- time integrators ----------------------------------------------------------------------
int klsa_dynamic_create(klsa_problem* prob, const char* method, int nonlinear, const klsa_options* opt,
                        klsa_dynamic** out) {
    if (!prob || !method || !out) return KLSA_INVALID_ARGUMENT;
    *out = nullptr;
    return guarded([&] {
        DynamicGPU::Method m;
        std::string s(method);
        if (s == "Newmark") m = DynamicGPU::Newmark;
        else if (s == "Bathe") m = DynamicGPU::Bathe;
        else if (s == "Wilson") m = DynamicGPU::Wilson;
        else if (s == "ExplicitEuler") m = DynamicGPU::ExplicitEuler;
        else if (s == "ImplicitEuler") m = DynamicGPU::ImplicitEuler;
        else if (s == "RK4") m = DynamicGPU::RK4;
        else {
            g_err = "unknown time integrator " + s;
            return KLSA_INVALID_ARGUMENT;
        }
        std::unique_ptr<klsa_dynamic> h(new klsa_dynamic);
        h->prob = prob;
        h->D.reset(new DynamicGPU(*prob->P, m, nonlinear != 0, opt ? opt->o : Options()));
        *out = h.release();
        return KLSA_SUCCESS;
    });
}
int klsa_dynamic_destroy(klsa_dynamic* d) {
    return guarded([&] {
        delete d;
        return KLSA_SUCCESS;
    });
}
int klsa_dynamic_set_load_table(klsa_dynamic* d, const double* t, const double* f, int n) {
    if (!d || n < 0 || (n > 0 && (!t || !f))) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        d->D->set_load_table(std::vector<double>(t, t + n), std::vector<double>(f, f + n));
        return KLSA_SUCCESS;
    });
}
int klsa_dynamic_set_state(klsa_dynamic* d, const double* U, const double* V, const double* A) {
    if (!d) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *d->prob->P;
        if (U) P.upload_pub(U, d->D->U());
        if (V) P.upload_pub(V, d->D->V());
        if (A) P.upload_pub(A, d->D->A());
        KL_CUDA(cudaStreamSynchronize(P.stream));
        return KLSA_SUCCESS;
    });
}
int klsa_dynamic_state(klsa_dynamic* d, double* U, double* V, double* A) {
    if (!d) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        Problem& P = *d->prob->P;
        if (U) P.download_pub(d->D->U(), U);
        if (V) P.download_pub(d->D->V(), V);
        if (A) P.download_pub(d->D->A(), A);
        return KLSA_SUCCESS;
    });
}
int klsa_dynamic_step(klsa_dynamic* d, double dt) {
    if (!d) return KLSA_INVALID_ARGUMENT;
    return guarded([&] { return d->D->step(dt > 0.0 ? dt : d->D->default_dt()); });
}
int klsa_dynamic_set_time(klsa_dynamic* d, double t) {
    if (!d) return KLSA_INVALID_ARGUMENT;
    d->D->set_time(t);
    return KLSA_SUCCESS;
}
double klsa_dynamic_time(klsa_dynamic* d) { return d ? d->D->time() : 0.0; }
int klsa_dynamic_iterations(klsa_dynamic* d) { return d ? d->D->iterations() : -1; }

}  // extern "C"

// ---- batched Newton ------------------------------------------------------------------------
extern "C" {

int klsa_batch_create(const klsa_patch_desc* descs, int n, klsa_batch** out) {
    if (!descs || n < 1 || !out) return KLSA_INVALID_ARGUMENT;
    *out = nullptr;
    return guarded([&] {
        std::vector<const klsa_patch_desc*> v(n);
        for (int i = 0; i < n; ++i) v[i] = descs + i;
        std::unique_ptr<klsa_batch> b(new klsa_batch);
        b->B.reset(new BatchedProblem(v));
        *out = b.release();
        return KLSA_SUCCESS;
    });
}

int klsa_batch_destroy(klsa_batch* b) {
    delete b;
    return KLSA_SUCCESS;
}

int klsa_batch_info(klsa_batch* b, double* out) {
    if (!b || !out) return KLSA_INVALID_ARGUMENT;
    out[0] = b->B->ninst;
    out[1] = b->B->nfree;
    out[2] = (double)b->B->nnz;
    out[3] = (double)b->B->mf->front_bytes();
    return KLSA_SUCCESS;
}

int64_t klsa_batch_instance_ndof(klsa_batch* b, int i) {
    if (!b || i < 0 || i >= b->B->ninst) return -1;
    return b->B->inst[i]->nfree;
}

int klsa_batch_autotune(klsa_batch* b, double* log, int cap) {
    if (!b) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        b->B->autotune();
        int rows = (int)b->B->tune_log.size() / 4;
        if (log)
            for (int r = 0; r < std::min(rows, cap); ++r)
                for (int c = 0; c < 4; ++c) log[4 * r + c] = b->B->tune_log[4 * r + c];
        return rows;
    });
}

int klsa_batch_newton_create(klsa_batch* b, const klsa_options* opt, klsa_batch_newton** out) {
    if (!b || !out) return KLSA_INVALID_ARGUMENT;
    *out = nullptr;
    return guarded([&] {
        Options o = opt ? opt->o : Options{};
        std::unique_ptr<klsa_batch_newton> s(new klsa_batch_newton);
        s->b = b;
        s->N.reset(new BatchedNewton(*b->B, o));
        *out = s.release();
        return KLSA_SUCCESS;
    });
}

int klsa_batch_newton_destroy(klsa_batch_newton* s) {
    delete s;
    return KLSA_SUCCESS;
}

int klsa_batch_newton_solve(klsa_batch_newton* s) {
    if (!s) return KLSA_INVALID_ARGUMENT;
    return guarded([&] { return s->N->solve(); });
}

int klsa_batch_newton_reset(klsa_batch_newton* s) {
    if (!s) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        s->N->reset();
        return KLSA_SUCCESS;
    });
}

int klsa_batch_newton_results(klsa_batch_newton* s, int* status, int* iterations) {
    if (!s) return KLSA_INVALID_ARGUMENT;
    const int n = s->b->B->ninst;
    for (int i = 0; i < n; ++i) {
        if (status) status[i] = s->N->status()[i];
        if (iterations) iterations[i] = s->N->iterations()[i];
    }
    return KLSA_SUCCESS;
}

int klsa_batch_newton_solution(klsa_batch_newton* s, int i, double* U) {
    if (!s || !U || i < 0 || i >= s->b->B->ninst) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        BatchedProblem& B = *s->b->B;
        Problem& P = *B.inst[i];
        KL_CUDA(cudaStreamSynchronize(B.stream));
        P.download_pub(s->N->U() + B.dof_off[i], U, 1);
        return KLSA_SUCCESS;
    });
}

int klsa_batch_sync(klsa_batch* b) {
    if (!b) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        KL_CUDA(cudaStreamSynchronize(b->B->stream));
        return KLSA_SUCCESS;
    });
}

int klsa_batch_event_record(klsa_batch* b, int slot) {
    if (!b || slot < 0 || slot >= 16) return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        if (!b->ev[slot]) KL_CUDA(cudaEventCreate(&b->ev[slot]));
        KL_CUDA(cudaEventRecord(b->ev[slot], b->B->stream));
        return KLSA_SUCCESS;
    });
}

int klsa_batch_event_elapsed(klsa_batch* b, int slot_a, int slot_b, float* ms) {
    if (!b || !ms || slot_a < 0 || slot_a >= 16 || slot_b < 0 || slot_b >= 16 || !b->ev[slot_a] || !b->ev[slot_b])
        return KLSA_INVALID_ARGUMENT;
    return guarded([&] {
        KL_CUDA(cudaEventSynchronize(b->ev[slot_b]));
        KL_CUDA(cudaEventElapsedTime(ms, b->ev[slot_a], b->ev[slot_b]));
        return KLSA_SUCCESS;
    });
}

}  // extern "C"
