// multifrontal.h -- nested-dissection multifrontal LDL^T on the device (FP32 or FP64 fronts).
//
// Stands in for the sparse factorisation behind the reference's "SimplicialLDLT" solver name
// (Eigen SimplicialLDLT via gsSparseSolver<T>::get, gsStaticSolvers/gsStaticBase.h:85,
// gsALMSolvers/gsALMBase.hpp:73-78): an LDL^T without pivoting, so it factorises the
// indefinite tangents met past limit points, and its D gives the determinant stability
// indicator (gsStaticBase.h:162-179).
//
// Layout in HBM: one pool of dense column-major fronts (f x f, ld = f, lower triangle used),
// per-node inverse diagonal tiles (64x64), per-node inverses X = L11^-1 of the own block (k x k,
// row-major), a double-buffered panel workspace W = L*D (f x 64), per-node solve update vectors.
// Work lists per (level, tile step, phase) are built once on the host.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "nd_symbolic.h"

namespace klsa {

// Per-level tile lists of the persistent triangular solve (offsets into the work-item pool):
// own = lower-triangular 64x64 tiles of X = L11^-1, halo = 64x64 tiles of L21.
constexpr int MF_MAX_LEVELS = 48;
struct SolveLevels {
    int nlev;
    int own_off[MF_MAX_LEVELS], own_cnt[MF_MAX_LEVELS], halo_off[MF_MAX_LEVELS], halo_cnt[MF_MAX_LEVELS];
};

constexpr int MF_NB = 64;          // tile size
constexpr int MF_MAX_RHS = 4;

struct MFWork {
    int4* items = nullptr;   // device pointer into the item pool
    int count = 0;
};

template <class T>
class MultifrontalT {
public:
    // csr (internal order): rowptr/cols on the host, used to build the front scatter map
    MultifrontalT(const NDTree& tree, const std::vector<int>& rowptr, const std::vector<int>& cols,
                 cudaStream_t stream);
    ~MultifrontalT();

    // Numeric factorisation of the FP32 CSR values (internal order, same pattern).
    // Returns ST_SUCCESS or ST_SOLVER_ERROR (zero / non-finite pivot).
    int factorize(const T* d_vals, bool check_status = true);
    // Enqueue the factorisation without the status read-back (status stays on the device).
    void factorize_async(const T* d_vals);
    int read_status();
    // x = (L D L^T)^-1 b for nrhs columns (ld = n), front precision in/out, internal order.
    void solve(const T* d_b, T* d_x, int nrhs);
    // min(D) and #negatives of D (after factorize)
    void stability(double* min_d, int64_t* negatives);
    // The launch sequences alone (no graph of their own), for callers that capture a larger
    // graph around them.
    void enqueue_factorize(const T* d_vals);
    void enqueue_solve(const T* d_b, T* d_x);

    int n() const { return n_; }
    // number of factorisations enqueued so far (identifies the factor the fronts hold)
    uint64_t generation() const { return generation_; }
    double flops() const { return flops_; }
    int64_t front_bytes() const { return (int64_t)pool_.size() * 4; }
    // algorithmic bytes / flops of one factorisation per kernel kind (0 diag, 1 panel, 2 update),
    // launches per factorisation, and bytes of one triangular solve (L read forward and backward)
    double kernel_bytes[3] = {0, 0, 0}, kernel_flops[3] = {0, 0, 0};
    int kernel_launches[3] = {0, 0, 0};
    double solve_bytes = 0;
    const std::vector<int>& level_nodes(int lvl) const { return level_nodes_[lvl]; }

private:
    uint64_t generation_ = 0;
    struct GraphSlot {
        cudaGraphExec_t exec = nullptr;
        const void* key0 = nullptr;
        const void* key1 = nullptr;
        unsigned long long kernels = 0;
    };
    template <class Fn> void replay(GraphSlot& slot, const void* key0, const void* key1, Fn&& launches);
    void factorize_launches(const T* d_vals);
    template <int NR> void solve_impl(const T* d_b, T* d_x);
    // one cooperative launch per solve (all levels, both sweeps); the five-launch-per-level
    // solve_impl stays for graph-captured callers and as the "levels" variant
    template <int NR> void solve_persistent(const T* d_b, T* d_x);
    bool persistent_solve_enabled() const;
    SolveLevels* solve_levels_ = nullptr;
    DevBuf<int64_t> d_inv_off_;
    DevBuf<int> d_inv_;
    int ps_grid_[3] = {0, 0, 0};
    // dataflow variant of the persistent solve (default; KLSA_SOLVE_KERNEL=barrier selects the
    // level-barrier kernel): queue of (phase, tile), tiles per node, completion counters
    DevBuf<int> df_queue_, df_own_t_, df_halo_t_, df_cnt_;
    DevBuf<T> df_r_;             // fan-out right-hand side (n x MF_MAX_RHS)
    int df_qtotal_ = 0;
    int df_grid_[3] = {0, 0, 0};
    int df_stall_node_ = -1;
    bool update_tc_ = false;     // trailing updates on the tensor cores (FP32 fronts, KLSA_UPDATE_KERNEL=tc)
    void launch_update(const MFWork& w, int t, const T* W, cudaStream_t s);     // test hook (KLSA_SOLVE_STALL_NODE=k): the k-th leaf's first phase never completes
    bool persistent_ok_ = true;
    size_t ps_smem_[3] = {0, 0, 0};
    GraphSlot fact_graph_, solve_graph_[3];
    cudaStream_t stream_;
    cudaStream_t side_ = nullptr;          // look-ahead stream of the off-critical-path updates
    cudaEvent_t ev_panel_ = nullptr, ev_rest_ = nullptr;
    int64_t ws_half_ = 0;                  // W is double-buffered by step parity
    int n_ = 0, nnodes_ = 0, nlevels_ = 0;
    double flops_ = 0;
    // per-node device metadata
    DevBuf<int> d_f_, d_k_, d_own_, d_parent_;
    DevBuf<int64_t> d_front_off_, d_linv_off_, d_ws_off_, d_upd_off_, d_halo_off_, d_map_off_, d_xinv_off_;
    DevBuf<int> d_child0_, d_child1_;
    DevBuf<int> d_halo_, d_map_;
    DevBuf<int64_t> d_fpos_;     // CSR nz -> pool position (lower entries) or -1
    int64_t nnz_ = 0;
    DevBuf<T> pool_, linv_, ws_, upd_, D_;
    DevBuf<T> y_, z_;        // solve intermediates (n x MF_MAX_RHS)
    DevBuf<T> xinv_;         // per-node X = L11^-1 (k x k, row-major)
    cudaStream_t inv_stream_ = nullptr;    // node inverses, overlapped with the next levels
    cudaEvent_t ev_level_ = nullptr, ev_inv_ = nullptr;
    DevBuf<int> status_;
    DevBuf<int4> items_;
    // update tiles of a step: the first column block of the trailing matrix (the next step's
    // pivots, on the critical path) and the rest (overlapped with the next diagonal and panel)
    struct Step { MFWork diag, panel, upd_next, upd_rest; int t; };
    struct Level {
        MFWork ea[2];
        std::vector<Step> steps;
        MFWork nodes;             // one item per node (solve gather)
        MFWork own_blocks;        // (node, 64-row block of the own part)
        MFWork halo_blocks;       // (node, 64-row block of the halo)
        std::vector<MFWork> xdiag; // per block row bi: (node, bi) diagonal block of X
        std::vector<MFWork> xoff;  // per block row bi: (node, bi, bj < bi), empty for bi = 0
        int max_f = 0, max_k = 0, max_h = 0;
    };
    std::vector<Level> levels_;
    std::vector<std::vector<int>> level_nodes_;
    int max_f_ = 0;
};

// FP32 fronts (inexact Newton corrector, preconditioned refinement) and FP64 fronts (operators
// that must be exact to FP64 working accuracy, e.g. the shift-invert eigen operators of large
// thin shells whose FP32 factor is too inaccurate for iterative refinement to converge).
using Multifrontal = MultifrontalT<float>;
using Multifrontal64 = MultifrontalT<double>;

}  // namespace klsa
