// batch.h -- many independent single-patch shells solved together on one GPU.
//
// The reference has no batched API: a user loops over gsStaticNewton instances, one
// assembler + sparse factorisation each (gsStaticSolvers/gsStaticNewton.hpp:142-193).  Here
// the instances share every launch:
//   * assembly: persistent kernels walk the flat element list of all instances of one degree
//     (per-instance tables, geometry and displacement reached through a descriptor array);
//   * factorisation: the nested-dissection trees of all instances form one elimination forest
//     whose levels are processed by the same per-level multifrontal launches as one patch
//     (the merged matrix is block diagonal, so the forest is exact);
//   * Newton control: per-instance norms, convergence tests and freezing of converged
//     instances run on the device; one CUDA graph replays a whole Newton iteration and the host
//     reads a single counter of unconverged instances per iteration.
#pragma once

#include <memory>
#include <vector>

#include "multifrontal.h"
#include "problem.h"
#include "solvers.h"

struct klsa_patch_desc;

namespace klsa {

// Per-instance view used by the batched kernels (lives in device memory).
struct BatchInst {
    const double* tab1;
    const double* tab2;
    const float2* tab1s;     // the same tables as FP32 hi/lo pairs (double-float internal force)
    const float2* tab2s;
    const double* qpgeo;
    double* ufull;
    float* elemK;
    double* elemR;
    const int* int2full;
    int p, nq, m1, m2, n1, ncp, nel, nfree;
    int dof_off;       // first row of the instance in the merged free-dof numbering
    double tm, tb;     // t and t^3/12
};

class BatchedProblem {
public:
    explicit BatchedProblem(const std::vector<const klsa_patch_desc*>& descs);
    ~BatchedProblem();

    int ninst = 0;
    std::vector<std::unique_ptr<Problem>> inst;
    cudaStream_t stream = nullptr;
    int nfree = 0;
    int64_t nnz = 0;
    std::vector<int> dof_off;            // ninst + 1
    std::vector<BatchInst> desc;
    DevBuf<BatchInst> d_desc;
    DevBuf<int> d_dof_off, d_dof_inst;
    struct DegreeList {
        int ninst = 0, nel = 0, ngrp = 0;
        DevBuf<int> insts, elem_off, grp_off;
    };
    DegreeList deg[2];                   // degree 2 and degree 3 instances
    DevBuf<int> d_rowptr, d_cols;        // merged block-diagonal CSR (internal order)
    DevBuf<float> d_vals32;
    DevBuf<double> d_F;                  // merged external load
    std::unique_ptr<Multifrontal> mf;
    int num_sms = 1;
    // blocks per SM of the persistent kernels, per degree; chosen by autotune()
    int tangent_bps[2] = {4, 4}, fint_bps[2] = {4, 4};
    bool tuned = false;
    std::vector<double> tune_log;        // (kind 0 tangent / 1 fint, degree, blocks per SM, ms) per trial

    void set_displacement(const double* d_x);   // merged free vector -> per-instance full vectors
    void tangent_f32();                          // K(u) of every instance -> d_vals32
    void internal_force(double* d_out);          // Fint(u) of every instance, merged
    void autotune();                             // time the persistent-kernel launch shapes

    // launchers implemented beside the element kernels
    void launch_tangent(int d, int bps);
    void launch_gather_K();
    void launch_fint(int d, int bps);
    void launch_gather_R(double* d_out);
};

// gsStaticNewton::solve() on every instance (gsStaticNewton.hpp:101-193): the first solve starts
// from a linear head start; convergence relax*|dU|/|DU| < tolU and |R|/|R0| < tolF per instance.
class BatchedNewton {
public:
    BatchedNewton(BatchedProblem& B, const Options& opt);
    ~BatchedNewton();
    int solve();
    void reset();   // U = 0 and a fresh head start for the next solve()
    const std::vector<int>& status() const { return status_; }
    const std::vector<int>& iterations() const { return iters_; }
    const double* U() const { return U_.get(); }
    int graph_kernels() const { return (int)graph_kernels_; }

private:
    void residual(const double* d_x, double* d_R);
    void iteration_launches();
    BatchedProblem& B_;
    double tolF_, tolU_, relax_, L_;
    int maxIt_, refine_ = 1;
    DevBuf<double> U_, DU_, dU_, R_, x_, fint_, norms_, resIni_;
    DevBuf<float> b32_, x32_;
    DevBuf<int> active_, fin_, st_, its_, it_, count_;
    int* h_count_ = nullptr;
    bool headstart_ = false;
    cudaGraphExec_t graph_ = nullptr;
    unsigned long long graph_kernels_ = 0;
    std::vector<int> status_, iters_;
};

}  // namespace klsa
