// batch.cu -- merged elimination forest, launch-shape autotuner and device-side Newton control
// for many independent patches (no counterpart in the reference, which runs one
// gsStaticNewton per patch: gsStaticSolvers/gsStaticNewton.hpp:101-193).
#include "batch.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <thread>

#include "../../include/klshell_gb300.h"
#include "linalg.h"

namespace klsa {

namespace {

// out[3k + c] = squared 2-norm of vector c (a, b, d) over the rows of instance k; one block per
// instance, fixed summation order.
__global__ void seg_norms_kernel(int ninst, const int* __restrict__ dof_off, const double* __restrict__ a,
                                 const double* __restrict__ b, const double* __restrict__ c, double* __restrict__ out) {
    __shared__ double red[3][8];
    const int k = blockIdx.x;
    const int r0 = dof_off[k], r1 = dof_off[k + 1];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        s0 += a[r] * a[r];
        s1 += b[r] * b[r];
        s2 += c[r] * c[r];
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[0][warp] = s0; red[1][warp] = s1; red[2][warp] = s2; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x][w];
        out[3 * k + threadIdx.x] = s;
    }
}

__global__ void init_state_kernel(int ninst, const double* __restrict__ norms, double* __restrict__ resIni,
                                  int* __restrict__ active, int* __restrict__ st, int* __restrict__ its,
                                  int* __restrict__ it, int* __restrict__ count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ninst) {
        double r = sqrt(norms[3 * k]);
        resIni[k] = (r == 0.0) ? 1.0 : r;
        active[k] = 1;
        st[k] = ST_NOT_STARTED;
        its[k] = 0;
    }
    if (k == 0) { it[0] = 0; count[0] = ninst; }
}

// Convergence test of gsStaticNewton::_solveNonlinear (gsStaticNewton.hpp:180-190) for every
// unconverged instance; converged (or out-of-iterations) instances are marked for finalising
// (U += DU) and leave the active set.
__global__ void newton_control_kernel(int ninst, const double* __restrict__ norms, const double* __restrict__ resIni,
                                      int* __restrict__ active, int* __restrict__ fin, int* __restrict__ st,
                                      int* __restrict__ its, int* __restrict__ it, int* __restrict__ count,
                                      double tolF, double tolU, double relax, int maxIt) {
    __shared__ int cnt;
    const int itv = it[0];
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    int local = 0;
    for (int k = threadIdx.x; k < ninst; k += blockDim.x) {
        fin[k] = 0;
        if (!active[k]) continue;
        const double res = sqrt(norms[3 * k]);
        const double ratioU = relax * sqrt(norms[3 * k + 1]) / sqrt(norms[3 * k + 2]);
        if (ratioU < tolU && res / resIni[k] < tolF) {
            fin[k] = 1; active[k] = 0; st[k] = ST_SUCCESS; its[k] = itv;
        } else if (itv + 1 == maxIt) {
            fin[k] = 1; active[k] = 0; st[k] = ST_NOT_CONVERGED; its[k] = itv;
        } else {
            ++local;
        }
    }
    atomicAdd(&cnt, local);
    __syncthreads();
    if (threadIdx.x == 0) {
        count[0] = cnt;
        it[0] = itv + 1;
    }
}

__global__ void finalize_kernel(int n, const int* __restrict__ dof_inst, const int* __restrict__ fin,
                                double* __restrict__ U, double* __restrict__ DU) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n && fin[dof_inst[r]]) {
        U[r] += DU[r];
        DU[r] = 0.0;
    }
}

// y = A x over the merged CSR (FP32 values, FP64 vectors), one warp per row
__global__ void csr_spmv_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ cols,
                                const float* __restrict__ vals, const double* __restrict__ x, double* __restrict__ y) {
    const int row = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    double s = 0.0;
    for (int z = rowptr[row] + lane; z < rowptr[row + 1]; z += 32) s += (double)vals[z] * x[cols[z]];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[row] = s;
}

__global__ void masked_axpy_kernel(int n, const int* __restrict__ dof_inst, const int* __restrict__ active, double a,
                                   const double* __restrict__ x, double* __restrict__ y) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n && active[dof_inst[r]]) y[r] += a * x[r];
}

}  // namespace

// ------------------------------------------------------------------------------------------
BatchedProblem::BatchedProblem(const std::vector<const klsa_patch_desc*>& descs) {
    ninst = (int)descs.size();
    if (ninst < 1) throw std::invalid_argument("batch needs at least one instance");
    for (const klsa_patch_desc* d : descs)
        if (!d || (d->p != 2 && d->p != 3)) throw std::invalid_argument("batched instances must have degree 2 or 3");
    inst.resize(ninst);
    // instances are independent: build them on all host threads
    {
        unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 16u));
        std::vector<std::thread> pool;
        std::vector<std::string> errs(nt);
        for (unsigned t = 0; t < nt; ++t)
            pool.emplace_back([&, t] {
                try {
                    for (int i = (int)t; i < ninst; i += (int)nt) inst[i].reset(new Problem(*descs[i]));
                } catch (const std::exception& e) {
                    errs[t] = e.what();
                }
            });
        for (auto& th : pool) th.join();
        for (const std::string& e : errs)
            if (!e.empty()) throw std::invalid_argument("batch instance: " + e);
    }
    KL_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    int dev = 0;
    KL_CUDA(cudaGetDevice(&dev));
    KL_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));

    // merged numbering, CSR, load and elimination forest
    dof_off.assign(ninst + 1, 0);
    int64_t tot = 0, totnz = 0;
    for (int i = 0; i < ninst; ++i) {
        dof_off[i] = (int)tot;
        tot += inst[i]->nfree;
        totnz += inst[i]->nnz;
    }
    if (tot >= (int64_t)1 << 31 || totnz >= (int64_t)1 << 31) throw std::invalid_argument("batch too large for int32 CSR");
    dof_off[ninst] = (int)tot;
    nfree = (int)tot;
    nnz = totnz;
    std::vector<int> rowptr(nfree + 1, 0), cols((size_t)nnz), dof_inst(nfree);
    std::vector<double> F(nfree);
    NDTree M;
    M.nfree = nfree;
    for (int i = 0; i < ninst; ++i) {
        const Problem& P = *inst[i];
        const int off = dof_off[i];
        const int64_t zoff = P.rowptr.empty() ? 0 : rowptr[off];
        for (int r = 0; r < P.nfree; ++r) {
            rowptr[off + r + 1] = (int)(zoff + P.rowptr[r + 1]);
            dof_inst[off + r] = i;
            F[off + r] = P.F_int_order[r];
        }
        for (int64_t z = 0; z < P.nnz; ++z) cols[zoff + z] = P.cols[z] + off;
        const int noff = (int)M.nodes.size();
        for (const NDNode& nd : P.tree.nodes) {
            NDNode c = nd;
            c.own_start += off;
            for (int& h : c.halo) h += off;
            if (c.parent >= 0) c.parent += noff;
            for (int& ch : c.child)
                if (ch >= 0) ch += noff;
            M.nodes.push_back(std::move(c));
        }
        for (int nd : P.tree.node_of) M.node_of.push_back(nd + noff);
        for (const auto& pm : P.tree.parent_map) M.parent_map.push_back(pm);
        M.max_height = std::max(M.max_height, P.tree.max_height);
    }
    d_rowptr.upload(rowptr, stream);
    d_cols.upload(cols, stream);
    d_vals32.alloc(std::max<int64_t>(nnz, 1));
    d_F.upload(F, stream);
    d_dof_off.upload(dof_off, stream);
    d_dof_inst.upload(dof_inst, stream);
    mf.reset(new Multifrontal(M, rowptr, cols, stream));

    // per-instance element buffers and descriptors; per-degree work lists
    desc.resize(ninst);
    std::vector<int> insts[2], eoff[2], goff[2];
    for (int d = 0; d < 2; ++d) { eoff[d].push_back(0); goff[d].push_back(0); }
    for (int i = 0; i < ninst; ++i) {
        Problem& P = *inst[i];
        const int D = 3 * (P.p + 1) * (P.p + 1);
        P.d_elemKf.alloc((size_t)P.nel * D * D);
        P.d_elemR.alloc((size_t)P.nel * D);
        BatchInst& b = desc[i];
        b.tab1 = P.d_tab1.get(); b.tab2 = P.d_tab2.get(); b.tab1s = P.d_tab1s.get(); b.tab2s = P.d_tab2s.get(); b.qpgeo = P.d_qpgeo.get(); b.ufull = P.d_ufull.get();
        b.elemK = P.d_elemKf.get(); b.elemR = P.d_elemR.get(); b.int2full = P.d_int2full.get();
        b.p = P.p; b.nq = P.nq; b.m1 = P.m1; b.m2 = P.m2; b.n1 = P.n1; b.ncp = P.ncp; b.nel = P.nel;
        b.nfree = P.nfree; b.dof_off = dof_off[i];
        b.tm = P.t; b.tb = P.t * P.t * P.t / 12.0;
        const int lpe = std::max((P.p + 1) * (P.p + 1), P.nq * P.nq);
        if (lpe > 32) throw std::invalid_argument("batched internal force: (p+1)^2 and nq^2 must be <= 32");
        const int es = 32 / lpe;
        const int d = P.p - 2;
        insts[d].push_back(i);
        eoff[d].push_back(eoff[d].back() + P.nel);
        goff[d].push_back(goff[d].back() + ceil_div(P.nel, es));
    }
    for (int d = 0; d < 2; ++d) {
        deg[d].ninst = (int)insts[d].size();
        deg[d].nel = eoff[d].back();
        deg[d].ngrp = goff[d].back();
        if (deg[d].ninst) {
            deg[d].insts.upload(insts[d], stream);
            deg[d].elem_off.upload(eoff[d], stream);
            deg[d].grp_off.upload(goff[d], stream);
        }
    }
    d_desc.upload(desc, stream);
    KL_CUDA(cudaStreamSynchronize(stream));
}

BatchedProblem::~BatchedProblem() {
    mf.reset();
    if (stream) cudaStreamDestroy(stream);
}

// Launch-shape autotuner of the persistent assembly kernels: every candidate number of resident
// blocks per SM is timed with CUDA events on the current displacement (best of three after one
// warm-up launch) and the fastest is kept per kernel and degree.
void BatchedProblem::autotune() {
    static const int cand[] = {1, 2, 3, 4, 6, 8, 12, 16};
    cudaEvent_t e0, e1;
    KL_CUDA(cudaEventCreate(&e0));
    KL_CUDA(cudaEventCreate(&e1));
    tune_log.clear();
    for (int kind = 0; kind < 2; ++kind)
        for (int d = 0; d < 2; ++d) {
            if (deg[d].ninst == 0) continue;
            double best = 1e30;
            int best_bps = 4;
            for (int bps : cand) {
                auto run = [&] { kind == 0 ? launch_tangent(d, bps) : launch_fint(d, bps); };
                run();
                float tmin = 1e30f;
                for (int rep = 0; rep < 3; ++rep) {
                    KL_CUDA(cudaEventRecord(e0, stream));
                    run();
                    KL_CUDA(cudaEventRecord(e1, stream));
                    KL_CUDA(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    KL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                    tmin = std::min(tmin, ms);
                }
                tune_log.insert(tune_log.end(), {(double)kind, (double)(d + 2), (double)bps, (double)tmin});
                if (tmin < best) { best = tmin; best_bps = bps; }
            }
            (kind == 0 ? tangent_bps : fint_bps)[d] = best_bps;
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tuned = true;
}

// ------------------------------------------------------------------------------------------
BatchedNewton::BatchedNewton(BatchedProblem& B, const Options& opt) : B_(B) {
    // gsStaticBase / gsStaticNewton defaults (gsStaticBase.h:66-75): tol 1e-6, maxIt 25
    double tol = opt.real("tol", 1e-6);
    tolF_ = opt.real("tolF", -1) != -1 ? opt.real("tolF", -1) : tol;
    tolU_ = opt.real("tolU", -1) != -1 ? opt.real("tolU", -1) : tol;
    maxIt_ = (int)opt.integer("maxIt", 25);
    refine_ = (int)opt.integer("Refinement", 1);
    relax_ = opt.real("Relaxation", 1.0);
    L_ = opt.real("LoadFactor", 1.0);
    if (maxIt_ < 1) throw std::invalid_argument("maxIt must be positive");
    const int n = B_.nfree, k = B_.ninst;
    for (DevBuf<double>* b : {&U_, &DU_, &dU_, &R_, &x_, &fint_}) {
        b->alloc(n);
        b->zero(B_.stream);
    }
    b32_.alloc(n);
    x32_.alloc(n);
    norms_.alloc(3 * (size_t)k);
    resIni_.alloc(k);
    for (DevBuf<int>* b : {&active_, &fin_, &st_, &its_}) {
        b->alloc(k);
        b->zero(B_.stream);
    }
    it_.alloc(1);
    count_.alloc(1);
    KL_CUDA(cudaMallocHost(&h_count_, sizeof(int)));
    status_.assign(k, ST_NOT_STARTED);
    iters_.assign(k, 0);
    if (!B_.tuned) B_.autotune();
    KL_CUDA(cudaStreamSynchronize(B_.stream));
}

BatchedNewton::~BatchedNewton() {
    if (graph_) cudaGraphExecDestroy(graph_);
    if (h_count_) cudaFreeHost(h_count_);
}

void BatchedNewton::reset() {
    U_.zero(B_.stream);
    DU_.zero(B_.stream);
}

void BatchedNewton::residual(const double* d_x, double* d_R) {
    // Residual_t convention R = L F - Fint (gsStructuralAnalysisTypes.h:70-76)
    B_.set_displacement(d_x);
    B_.internal_force(fint_.get());
    vec::lincomb(L_, B_.d_F.get(), -1.0, fint_.get(), d_R, B_.nfree, B_.stream);
}

// One Newton iteration of every active instance (gsStaticNewton.hpp:157-190).
void BatchedNewton::iteration_launches() {
    const int n = B_.nfree;
    cudaStream_t s = B_.stream;
    vec::lincomb(1.0, U_.get(), 1.0, DU_.get(), x_.get(), n, s);
    B_.set_displacement(x_.get());
    B_.tangent_f32();
    B_.mf->enqueue_factorize(B_.d_vals32.get());
    vec::to_f32(R_.get(), b32_.get(), n, s);
    B_.mf->enqueue_solve(b32_.get(), x32_.get());
    vec::to_f64(x32_.get(), dU_.get(), n, s);
    // iterative refinement of the Newton step against the assembled (FP32) tangent: removes most
    // of the FP32 factorisation error, so thin, ill-conditioned panels converge in a few steps
    for (int r = 0; r < refine_; ++r) {
        csr_spmv_kernel<<<ceil_div((int64_t)n * 32, 256), 256, 0, s>>>(n, B_.d_rowptr.get(), B_.d_cols.get(),
                                                                      B_.d_vals32.get(), dU_.get(), x_.get());
        count_launch();
        vec::lincomb(1.0, R_.get(), -1.0, x_.get(), x_.get(), n, s);
        vec::to_f32(x_.get(), b32_.get(), n, s);
        B_.mf->enqueue_solve(b32_.get(), x32_.get());
        vec::to_f64(x32_.get(), x_.get(), n, s);
        vec::axpby(1.0, x_.get(), 1.0, dU_.get(), n, s);
    }
    masked_axpy_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, B_.d_dof_inst.get(), active_.get(), relax_, dU_.get(),
                                                       DU_.get());
    count_launch();
    vec::lincomb(1.0, U_.get(), 1.0, DU_.get(), x_.get(), n, s);
    residual(x_.get(), R_.get());
    seg_norms_kernel<<<B_.ninst, 256, 0, s>>>(B_.ninst, B_.d_dof_off.get(), R_.get(), dU_.get(), DU_.get(),
                                             norms_.get());
    count_launch();
    newton_control_kernel<<<1, 256, 0, s>>>(B_.ninst, norms_.get(), resIni_.get(), active_.get(), fin_.get(),
                                           st_.get(), its_.get(), it_.get(), count_.get(), tolF_, tolU_, relax_,
                                           maxIt_);
    count_launch();
    finalize_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, B_.d_dof_inst.get(), fin_.get(), U_.get(), DU_.get());
    count_launch();
    KL_CUDA(cudaMemcpyAsync(h_count_, count_.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
    KL_CHECK_LAUNCH();
}

int BatchedNewton::solve() {
    const int n = B_.nfree;
    cudaStream_t s = B_.stream;
    // No linear head start: after gsStaticBase::initialize() (what the reference's drivers call)
    // m_DeltaU has the dofs' rows, so gsStaticNewton.hpp:148-153 never takes it.
    // _start (gsStaticNewton.hpp:274-316): R0 = R(U); with the head start the iteration begins at
    // U + DU, otherwise DU = 0
    if (!headstart_) DU_.zero(s);
    residual(U_.get(), R_.get());
    seg_norms_kernel<<<B_.ninst, 256, 0, s>>>(B_.ninst, B_.d_dof_off.get(), R_.get(), R_.get(), R_.get(),
                                             norms_.get());
    count_launch();
    init_state_kernel<<<ceil_div(B_.ninst, 256), 256, 0, s>>>(B_.ninst, norms_.get(), resIni_.get(), active_.get(),
                                                             st_.get(), its_.get(), it_.get(), count_.get());
    count_launch();
    if (headstart_) {
        vec::lincomb(1.0, U_.get(), 1.0, DU_.get(), x_.get(), n, s);
        residual(x_.get(), R_.get());
        headstart_ = false;
    }
    dU_.zero(s);
    if (!graph_) {
        CaptureCount cc;
        KL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
            iteration_launches();
        } catch (...) {
            cudaGraph_t g;
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        cudaGraph_t g;
        KL_CUDA(cudaStreamEndCapture(s, &g));
        KL_CUDA(cudaGraphInstantiate(&graph_, g, 0));
        cudaGraphDestroy(g);
        graph_kernels_ = cc.n;
    }
    for (int it = 0; it < maxIt_; ++it) {
        KL_CUDA(cudaGraphLaunch(graph_, s));
        count_launch(graph_kernels_);
        KL_CUDA(cudaStreamSynchronize(s));
        if (*h_count_ == 0) break;
    }
    const int fact_status = B_.mf->read_status();
    KL_CUDA(cudaMemcpyAsync(status_.data(), st_.get(), sizeof(int) * B_.ninst, cudaMemcpyDeviceToHost, s));
    KL_CUDA(cudaMemcpyAsync(iters_.data(), its_.get(), sizeof(int) * B_.ninst, cudaMemcpyDeviceToHost, s));
    KL_CUDA(cudaStreamSynchronize(s));
    bool all = true;
    for (int& st : status_) {
        if (st != ST_SUCCESS && fact_status != ST_SUCCESS) st = ST_SOLVER_ERROR;
        all = all && st == ST_SUCCESS;
    }
    return all ? ST_SUCCESS : ST_NOT_CONVERGED;
}

}  // namespace klsa
