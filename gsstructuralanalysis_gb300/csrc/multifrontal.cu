// multifrontal.cu -- numeric nested-dissection multifrontal LDL^T and triangular solves.
//
// Per level of the elimination tree (leaves first):
//   1. extend-add of the children's Schur complements into the parent fronts (one launch
//      per child slot, so sibling updates never race and the sum order is fixed);
//   2. per 64-column tile step of the pivots: diagonal LDL^T + explicit inverse of the unit
//      lower tile (one CTA per front), panel L21 = A21 L11^-T D^-1 and W = L21 D (one CTA per
//      64-row block), trailing lower update A22 -= W L21^T (one CTA per 64x64 tile).
// No pivoting (as Eigen's SimplicialLDLT); a zero or non-finite pivot sets the status word.
#include "multifrontal.h"

#include <algorithm>
#include <cmath>

namespace klsa {

namespace {

constexpr int NB = MF_NB;

__global__ void mf_scatter_kernel(int64_t nnz, const int64_t* __restrict__ fpos, const float* __restrict__ vals,
                                  float* __restrict__ pool) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nnz) {
        int64_t p = fpos[i];
        if (p >= 0) pool[p] = vals[i];
    }
}

__global__ void mf_extend_add_kernel(const int4* __restrict__ items, const int* __restrict__ f, const int* __restrict__ k,
                                     const int* __restrict__ parent, const int64_t* __restrict__ front_off,
                                     const int64_t* __restrict__ map_off, const int* __restrict__ map, float* pool) {
    int4 it = items[blockIdx.x];
    int c = it.x, a0 = it.y;
    int fc = f[c], kc = k[c], hc = fc - kc;
    int par = parent[c];
    int fp = f[par];
    const int* mp = map + map_off[c];
    const float* src = pool + front_off[c];
    float* dst = pool + front_off[par];
    int a1 = min(a0 + 32, hc);
    for (int a = a0; a < a1; ++a) {
        int pa = mp[a];
        const float* scol = src + (int64_t)(kc + a) * fc + kc;
        float* dcol = dst + (int64_t)pa * fp;
        for (int b = a + threadIdx.x; b < hc; b += blockDim.x) dcol[mp[b]] += scol[b];
    }
}

// Diagonal tile: LDL^T in shared memory, then the inverse of the unit lower factor.
__global__ void __launch_bounds__(256) mf_diag_kernel(const int4* __restrict__ items, int t, const int* __restrict__ f,
                                                      const int* __restrict__ k, const int* __restrict__ own,
                                                      const int64_t* __restrict__ front_off,
                                                      const int64_t* __restrict__ linv_off, float* pool, float* linv,
                                                      float* Dvec, int* status) {
    __shared__ float A[NB][NB + 1];
    __shared__ float X[NB][NB + 1];
    __shared__ float red[4][NB];
    int nd = items[blockIdx.x].x;
    int fN = f[nd], kN = k[nd];
    int c0 = t * NB;
    int kk = min(NB, kN - c0);
    float* F = pool + front_off[nd];
    int tx = threadIdx.x & (NB - 1), ty = threadIdx.x >> 6;
    for (int c = ty; c < NB; c += 4) {
        float v = 0.f;
        if (tx < kk && c < kk && tx >= c) v = F[(int64_t)(c0 + c) * fN + c0 + tx];
        A[tx][c] = v;
    }
    const int r = tx;
    bool bad = false;
    for (int j = 0; j < kk; ++j) {
        __syncthreads();
        float d = A[j][j];
        if (!(fabsf(d) > 0.f) || !isfinite(d)) { bad = true; d = 1.f; }
        float dinv = 1.f / d;
        float lrj = (r > j && r < kk) ? A[r][j] : 0.f;
        if (r < kk)
            for (int c = j + 1 + ty; c <= r; c += 4) A[r][c] -= lrj * A[c][j] * dinv;
        __syncthreads();
        if (ty == 0 && r > j && r < kk) A[r][j] = lrj * dinv;
    }
    __syncthreads();
    if (bad && threadIdx.x == 0) atomicExch(status, 1);
    // write back L (strict lower) and D (diagonal)
    for (int c = ty; c < kk; c += 4)
        if (tx < kk && tx >= c) F[(int64_t)(c0 + c) * fN + c0 + tx] = A[tx][c];
    if (ty == 0 && tx < kk) Dvec[own[nd] + c0 + tx] = A[tx][tx];
    // X = L^-1 (unit lower), row by row: X[r][c] = -sum_{m=c}^{r-1} L[r][m] X[m][c]
    for (int c = ty; c < NB; c += 4) X[tx][c] = (tx == c && tx < kk) ? 1.f : 0.f;
    for (int rr = 1; rr < kk; ++rr) {
        __syncthreads();
        int c = tx;
        float s = 0.f;
        if (c < rr)
            for (int m = c + ty; m < rr; m += 4) s += A[rr][m] * X[m][c];
        red[ty][c] = s;
        __syncthreads();
        if (ty == 0 && c < rr) X[rr][c] = -(red[0][c] + red[1][c] + red[2][c] + red[3][c]);
    }
    __syncthreads();
    float* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
    for (int rr = ty; rr < NB; rr += 4) Li[rr * NB + tx] = X[rr][tx];
}

// Panel: W = A21 * Linv^T (rows r0..r0+63), L21 = W D^-1 written in place, W kept for the update.
__global__ void __launch_bounds__(256) mf_panel_kernel(const int4* __restrict__ items, int t, const int* __restrict__ f,
                                                       const int* __restrict__ k, const int64_t* __restrict__ front_off,
                                                       const int64_t* __restrict__ linv_off,
                                                       const int64_t* __restrict__ ws_off, float* pool,
                                                       const float* __restrict__ linv, float* ws) {
    __shared__ float As[NB][NB + 1];   // As[m][rr] = A21[r0+rr][c0+m]
    __shared__ float Ls[NB][NB + 1];   // Ls[m][j]  = Linv[j][m]
    __shared__ float Dinv[NB];
    int4 it = items[blockIdx.x];
    int nd = it.x, r0 = it.y;
    int fN = f[nd], kN = k[nd];
    int c0 = t * NB;
    int kk = min(NB, kN - c0);
    float* F = pool + front_off[nd];
    const float* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
    int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    int lt = threadIdx.x & 63, lg = threadIdx.x >> 6;
    for (int m = lg; m < NB; m += 4) {
        int rr = lt;
        As[m][rr] = (m < kk && r0 + rr < fN) ? F[(int64_t)(c0 + m) * fN + r0 + rr] : 0.f;
        Ls[m][rr] = (m < kk && rr < kk) ? Li[rr * NB + m] : 0.f;
    }
    if (threadIdx.x < NB) {
        int j = threadIdx.x;
        Dinv[j] = (j < kk) ? 1.f / F[(int64_t)(c0 + j) * fN + c0 + j] : 0.f;
    }
    __syncthreads();
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[i][q] = 0.f;
    for (int m = 0; m < kk; ++m) {
        float a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[m][tx + 16 * i];
#pragma unroll
        for (int q = 0; q < 4; ++q) b[q] = Ls[m][ty + 16 * q];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = fmaf(a[i], b[q], acc[i][q]);
    }
    float* W = ws + ws_off[nd];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int j = ty + 16 * q;
        if (j >= kk) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int r = r0 + tx + 16 * i;
            if (r >= fN) continue;
            W[(int64_t)j * fN + r] = acc[i][q];
            F[(int64_t)(c0 + j) * fN + r] = acc[i][q] * Dinv[j];
        }
    }
}

// Trailing update of one 64x64 lower tile: A[R, C] -= W[R, :] L[C, :]^T.
__global__ void __launch_bounds__(256) mf_update_kernel(const int4* __restrict__ items, int t, const int* __restrict__ f,
                                                        const int* __restrict__ k, const int64_t* __restrict__ front_off,
                                                        const int64_t* __restrict__ ws_off, float* pool,
                                                        const float* __restrict__ ws) {
    __shared__ float Ws[NB][NB + 1];   // Ws[m][rr] = W[R0+rr][m]
    __shared__ float Ls[NB][NB + 1];   // Ls[m][cc] = L[C0+cc][c0+m]
    int4 it = items[blockIdx.x];
    int nd = it.x;
    int fN = f[nd], kN = k[nd];
    int c0 = t * NB;
    int kk = min(NB, kN - c0);
    int c1 = c0 + kk;
    int R0 = c1 + it.y * NB, C0 = c1 + it.z * NB;
    float* F = pool + front_off[nd];
    const float* W = ws + ws_off[nd];
    int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    int lt = threadIdx.x & 63, lg = threadIdx.x >> 6;
    for (int m = lg; m < NB; m += 4) {
        Ws[m][lt] = (m < kk && R0 + lt < fN) ? W[(int64_t)m * fN + R0 + lt] : 0.f;
        Ls[m][lt] = (m < kk && C0 + lt < fN) ? F[(int64_t)(c0 + m) * fN + C0 + lt] : 0.f;
    }
    __syncthreads();
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[i][q] = 0.f;
    for (int m = 0; m < kk; ++m) {
        float a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = Ws[m][tx + 16 * i];
#pragma unroll
        for (int q = 0; q < 4; ++q) b[q] = Ls[m][ty + 16 * q];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = fmaf(a[i], b[q], acc[i][q]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int C = C0 + ty + 16 * q;
        if (C >= fN) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int R = R0 + tx + 16 * i;
            if (R >= fN || R < C) continue;
            F[(int64_t)C * fN + R] -= acc[i][q];
        }
    }
}

// Forward substitution of one node: children's update vectors, unit-lower solve of the own
// block, update vector of the halo.  y holds the result in internal order.
__global__ void __launch_bounds__(256) mf_fwd_kernel(const int4* __restrict__ items, int n, int nrhs,
                                                     const int* __restrict__ f, const int* __restrict__ k,
                                                     const int* __restrict__ own, const int* __restrict__ child0,
                                                     const int* __restrict__ child1,
                                                     const int64_t* __restrict__ front_off,
                                                     const int64_t* __restrict__ linv_off,
                                                     const int64_t* __restrict__ upd_off,
                                                     const int64_t* __restrict__ map_off, const int* __restrict__ map,
                                                     const float* __restrict__ pool, const float* __restrict__ linv,
                                                     float* upd, const float* __restrict__ b, float* y) {
    extern __shared__ float rhs[];   // fN * nrhs
    __shared__ float yt[NB * MF_MAX_RHS];
    int nd = items[blockIdx.x].x;
    int fN = f[nd], kN = k[nd], hN = fN - kN, o = own[nd];
    const float* F = pool + front_off[nd];
    for (int q = 0; q < nrhs; ++q)
        for (int r = threadIdx.x; r < fN; r += blockDim.x) rhs[r + fN * q] = (r < kN) ? b[o + r + (int64_t)n * q] : 0.f;
    __syncthreads();
    int chs[2] = {child0[nd], child1[nd]};
    for (int s = 0; s < 2; ++s) {
        int c = chs[s];
        if (c >= 0) {
            int hc = f[c] - k[c];
            const int* mp = map + map_off[c];
            const float* u = upd + upd_off[c];
            for (int q = 0; q < nrhs; ++q)
                for (int a = threadIdx.x; a < hc; a += blockDim.x) rhs[mp[a] + fN * q] += u[a + hc * q];
        }
        __syncthreads();
    }
    int ntiles = (kN + NB - 1) / NB;
    for (int t = 0; t < ntiles; ++t) {
        int c0 = t * NB, kk = min(NB, kN - c0);
        const float* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
        for (int e = threadIdx.x; e < kk * nrhs; e += blockDim.x) {
            int j = e % kk, q = e / kk;
            float s = 0.f;
            for (int m = 0; m <= j; ++m) s += Li[j * NB + m] * rhs[c0 + m + fN * q];
            yt[j + NB * q] = s;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < kk * nrhs; e += blockDim.x) {
            int j = e % kk, q = e / kk;
            rhs[c0 + j + fN * q] = yt[j + NB * q];
        }
        __syncthreads();
        for (int r = c0 + kk + threadIdx.x; r < fN; r += blockDim.x) {
            float s[MF_MAX_RHS] = {0.f, 0.f, 0.f, 0.f};
            for (int j = 0; j < kk; ++j) {
                float l = F[(int64_t)(c0 + j) * fN + r];
                for (int q = 0; q < nrhs; ++q) s[q] += l * yt[j + NB * q];
            }
            for (int q = 0; q < nrhs; ++q) rhs[r + fN * q] -= s[q];
        }
        __syncthreads();
    }
    float* u = upd + upd_off[nd];
    for (int q = 0; q < nrhs; ++q) {
        for (int r = threadIdx.x; r < kN; r += blockDim.x) y[o + r + (int64_t)n * q] = rhs[r + fN * q];
        for (int a = threadIdx.x; a < hN; a += blockDim.x) u[a + hN * q] = rhs[kN + a + fN * q];
    }
}

// Backward substitution of one node: x_own = L11^-T (D^-1 y_own - L21^T x_halo).
__global__ void __launch_bounds__(256) mf_bwd_kernel(const int4* __restrict__ items, int n, int nrhs,
                                                     const int* __restrict__ f, const int* __restrict__ k,
                                                     const int* __restrict__ own,
                                                     const int64_t* __restrict__ front_off,
                                                     const int64_t* __restrict__ linv_off,
                                                     const int64_t* __restrict__ halo_off, const int* __restrict__ halo,
                                                     const float* __restrict__ pool, const float* __restrict__ linv,
                                                     const float* __restrict__ Dvec, const float* __restrict__ y,
                                                     float* x) {
    extern __shared__ float xs[];   // fN * nrhs
    __shared__ float zt[NB * MF_MAX_RHS];
    int nd = items[blockIdx.x].x;
    int fN = f[nd], kN = k[nd], hN = fN - kN, o = own[nd];
    const float* F = pool + front_off[nd];
    const int* hl = halo + halo_off[nd];
    for (int q = 0; q < nrhs; ++q) {
        for (int a = threadIdx.x; a < hN; a += blockDim.x) xs[kN + a + fN * q] = x[hl[a] + (int64_t)n * q];
        for (int r = threadIdx.x; r < kN; r += blockDim.x) xs[r + fN * q] = y[o + r + (int64_t)n * q] / Dvec[o + r];
    }
    __syncthreads();
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    int ntiles = (kN + NB - 1) / NB;
    for (int t = ntiles - 1; t >= 0; --t) {
        int c0 = t * NB, kk = min(NB, kN - c0), c1 = c0 + kk;
        for (int j = warp; j < kk; j += nwarp) {
            const float* col = F + (int64_t)(c0 + j) * fN;
            float s[MF_MAX_RHS] = {0.f, 0.f, 0.f, 0.f};
            for (int r = c1 + lane; r < fN; r += 32) {
                float l = col[r];
                for (int q = 0; q < nrhs; ++q) s[q] += l * xs[r + fN * q];
            }
            for (int q = 0; q < nrhs; ++q) {
                float v = s[q];
                for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
                if (lane == 0) zt[j + NB * q] = xs[c0 + j + fN * q] - v;
            }
        }
        __syncthreads();
        const float* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
        for (int e = threadIdx.x; e < kk * nrhs; e += blockDim.x) {
            int j = e % kk, q = e / kk;
            float s = 0.f;
            for (int m = j; m < kk; ++m) s += Li[m * NB + j] * zt[m + NB * q];
            xs[c0 + j + fN * q] = s;
        }
        __syncthreads();
    }
    for (int q = 0; q < nrhs; ++q)
        for (int r = threadIdx.x; r < kN; r += blockDim.x) x[o + r + (int64_t)n * q] = xs[r + fN * q];
}

__global__ void mf_stability_kernel(int n, const float* __restrict__ D, double* out_min, unsigned long long* out_neg) {
    __shared__ double smin[256];
    __shared__ unsigned long long sneg[256];
    double mn = 1e300;
    unsigned long long ng = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d = D[i];
        mn = d < mn ? d : mn;
        ng += d < 0 ? 1ull : 0ull;
    }
    smin[threadIdx.x] = mn;
    sneg[threadIdx.x] = ng;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + s]);
            sneg[threadIdx.x] += sneg[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out_min[blockIdx.x] = smin[0];
        out_neg[blockIdx.x] = sneg[0];
    }
}

}  // namespace

Multifrontal::Multifrontal(const NDTree& T, const std::vector<int>& rowptr, const std::vector<int>& cols,
                           cudaStream_t stream)
    : stream_(stream) {
    n_ = T.nfree;
    nnodes_ = (int)T.nodes.size();
    flops_ = T.factor_flops();
    std::vector<int> f(nnodes_), k(nnodes_), own(nnodes_), parent(nnodes_), c0(nnodes_), c1(nnodes_);
    std::vector<int64_t> front_off(nnodes_), linv_off(nnodes_), ws_off(nnodes_), upd_off(nnodes_),
        halo_off(nnodes_), map_off(nnodes_);
    std::vector<int> halo_all, map_all;
    int64_t fo = 0, lo = 0, wo = 0, uo = 0;
    for (int i = 0; i < nnodes_; ++i) {
        const NDNode& nd = T.nodes[i];
        f[i] = nd.f(); k[i] = nd.k; own[i] = nd.own_start; parent[i] = nd.parent;
        c0[i] = nd.child[0]; c1[i] = nd.child[1];
        front_off[i] = fo; fo += (int64_t)f[i] * f[i];
        linv_off[i] = lo; lo += (int64_t)((nd.k + NB - 1) / NB) * NB * NB;
        ws_off[i] = wo; wo += (int64_t)f[i] * NB;
        upd_off[i] = uo; uo += (int64_t)nd.h() * MF_MAX_RHS;
        halo_off[i] = (int64_t)halo_all.size();
        halo_all.insert(halo_all.end(), nd.halo.begin(), nd.halo.end());
        map_off[i] = (int64_t)map_all.size();
        map_all.insert(map_all.end(), T.parent_map[i].begin(), T.parent_map[i].end());
        max_f_ = std::max(max_f_, f[i]);
    }
    // CSR lower entries -> front positions
    nnz_ = cols.size();
    std::vector<int64_t> fpos(nnz_, -1);
    for (int R = 0; R < n_; ++R)
        for (int e = rowptr[R]; e < rowptr[R + 1]; ++e) {
            int C = cols[e];
            if (C > R) continue;
            int nd = T.node_of[C];
            int lc = C - T.nodes[nd].own_start;
            int lr = T.local_index(nd, R);
            if (lr < 0) throw std::logic_error("multifrontal: matrix entry outside its front");
            fpos[e] = front_off[nd] + (int64_t)lc * f[nd] + lr;
        }
    // levels and work lists
    nlevels_ = T.max_height + 1;
    level_nodes_.assign(nlevels_, {});
    for (int i = 0; i < nnodes_; ++i) level_nodes_[T.nodes[i].height].push_back(i);
    std::vector<int4> items;
    struct Pending { int level, kind, slot, step; size_t begin, end; };
    std::vector<Pending> marks;
    levels_.assign(nlevels_, {});
    for (int L = 0; L < nlevels_; ++L) {
        const auto& ln = level_nodes_[L];
        for (int slot = 0; slot < 2; ++slot) {
            size_t b = items.size();
            for (int nd : ln) {
                int c = slot == 0 ? c0[nd] : c1[nd];
                if (c < 0) continue;
                int hc = f[c] - k[c];
                for (int a0 = 0; a0 < hc; a0 += 32) items.push_back(make_int4(c, a0, 0, 0));
            }
            marks.push_back({L, 0, slot, 0, b, items.size()});
        }
        int maxt = 0;
        for (int nd : ln) maxt = std::max(maxt, (k[nd] + NB - 1) / NB);
        levels_[L].steps.resize(maxt);
        for (int t = 0; t < maxt; ++t) {
            levels_[L].steps[t].t = t;
            size_t b = items.size();
            for (int nd : ln)
                if (k[nd] > t * NB) items.push_back(make_int4(nd, t, 0, 0));
            marks.push_back({L, 1, 0, t, b, items.size()});
            b = items.size();
            for (int nd : ln) {
                if (k[nd] <= t * NB) continue;
                int cc1 = t * NB + std::min(NB, k[nd] - t * NB);
                for (int r0 = cc1; r0 < f[nd]; r0 += NB) items.push_back(make_int4(nd, r0, 0, 0));
            }
            marks.push_back({L, 2, 0, t, b, items.size()});
            b = items.size();
            for (int nd : ln) {
                if (k[nd] <= t * NB) continue;
                int cc1 = t * NB + std::min(NB, k[nd] - t * NB);
                int ntr = (f[nd] - cc1 + NB - 1) / NB;
                for (int ti = 0; ti < ntr; ++ti)
                    for (int tj = 0; tj <= ti; ++tj) items.push_back(make_int4(nd, ti, tj, 0));
            }
            marks.push_back({L, 3, 0, t, b, items.size()});
        }
        size_t b = items.size();
        for (int nd : ln) items.push_back(make_int4(nd, 0, 0, 0));
        marks.push_back({L, 4, 0, 0, b, items.size()});
        for (int nd : ln) levels_[L].max_f = std::max(levels_[L].max_f, f[nd]);
    }
    items_.upload(items, stream_);
    for (const Pending& m : marks) {
        MFWork w{items_.get() + m.begin, (int)(m.end - m.begin)};
        Level& lv = levels_[m.level];
        switch (m.kind) {
            case 0: lv.ea[m.slot] = w; break;
            case 1: lv.steps[m.step].diag = w; break;
            case 2: lv.steps[m.step].panel = w; break;
            case 3: lv.steps[m.step].update = w; break;
            default: lv.nodes = w; break;
        }
    }
    d_f_.upload(f, stream_); d_k_.upload(k, stream_); d_own_.upload(own, stream_); d_parent_.upload(parent, stream_);
    d_child0_.upload(c0, stream_); d_child1_.upload(c1, stream_);
    d_front_off_.upload(front_off, stream_); d_linv_off_.upload(linv_off, stream_); d_ws_off_.upload(ws_off, stream_);
    d_upd_off_.upload(upd_off, stream_); d_halo_off_.upload(halo_off, stream_); d_map_off_.upload(map_off, stream_);
    d_halo_.upload(halo_all, stream_); d_map_.upload(map_all, stream_);
    d_fpos_.upload(fpos, stream_);
    pool_.alloc(std::max<int64_t>(fo, 1));
    linv_.alloc(std::max<int64_t>(lo, 1));
    ws_.alloc(std::max<int64_t>(wo, 1));
    upd_.alloc(std::max<int64_t>(uo, 1));
    D_.alloc(std::max(n_, 1));
    y_.alloc((size_t)std::max(n_, 1) * MF_MAX_RHS);
    status_.alloc(1);
    status_.zero(stream_);
    size_t smem = (size_t)max_f_ * MF_MAX_RHS * sizeof(float);
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(smem, 48 * 1024)));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(smem, 48 * 1024)));
    KL_CUDA(cudaStreamSynchronize(stream_));
}

void Multifrontal::factorize_async(const float* d_vals) {
    if (!d_vals && nnz_ > 0) throw std::logic_error("multifrontal: no matrix values");
    KL_CUDA(cudaMemsetAsync(pool_.get(), 0, pool_.size() * sizeof(float), stream_));
    KL_CUDA(cudaMemsetAsync(status_.get(), 0, sizeof(int), stream_));
    if (nnz_ > 0) {
        mf_scatter_kernel<<<ceil_div(nnz_, 256), 256, 0, stream_>>>(nnz_, d_fpos_.get(), d_vals, pool_.get());
        count_launch();
    }
    for (int L = 0; L < nlevels_; ++L) {
        Level& lv = levels_[L];
        for (int s = 0; s < 2; ++s)
            if (lv.ea[s].count) {
                mf_extend_add_kernel<<<lv.ea[s].count, 128, 0, stream_>>>(lv.ea[s].items, d_f_.get(), d_k_.get(),
                                                                          d_parent_.get(), d_front_off_.get(),
                                                                          d_map_off_.get(), d_map_.get(), pool_.get());
                count_launch();
            }
        for (Step& st : lv.steps) {
            if (st.diag.count) {
                cudaEvent_t evk = g_timer.begin(stream_);
                mf_diag_kernel<<<st.diag.count, 256, 0, stream_>>>(st.diag.items, st.t, d_f_.get(), d_k_.get(),
                                                                   d_own_.get(), d_front_off_.get(), d_linv_off_.get(),
                                                                   pool_.get(), linv_.get(), D_.get(), status_.get());
                g_timer.end(stream_, 5, evk);
                count_launch();
            }
            if (st.panel.count) {
                cudaEvent_t evk = g_timer.begin(stream_);
                mf_panel_kernel<<<st.panel.count, 256, 0, stream_>>>(st.panel.items, st.t, d_f_.get(), d_k_.get(),
                                                                     d_front_off_.get(), d_linv_off_.get(),
                                                                     d_ws_off_.get(), pool_.get(), linv_.get(), ws_.get());
                g_timer.end(stream_, 6, evk);
                count_launch();
            }
            if (st.update.count) {
                cudaEvent_t evk = g_timer.begin(stream_);
                mf_update_kernel<<<st.update.count, 256, 0, stream_>>>(st.update.items, st.t, d_f_.get(), d_k_.get(),
                                                                       d_front_off_.get(), d_ws_off_.get(), pool_.get(),
                                                                       ws_.get());
                g_timer.end(stream_, 4, evk);
                count_launch();
            }
        }
    }
    KL_CHECK_LAUNCH();
}

int Multifrontal::read_status() {
    int st = 0;
    KL_CUDA(cudaMemcpyAsync(&st, status_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
    KL_CUDA(cudaStreamSynchronize(stream_));
    return st ? ST_SOLVER_ERROR : ST_SUCCESS;
}

int Multifrontal::factorize(const float* d_vals, bool check_status) {
    factorize_async(d_vals);
    return check_status ? read_status() : ST_SUCCESS;
}

void Multifrontal::solve(const float* d_b, float* d_x, int nrhs) {
    if (nrhs < 1 || nrhs > MF_MAX_RHS) throw std::invalid_argument("multifrontal solve: nrhs out of range");
    for (int L = 0; L < nlevels_; ++L) {
        Level& lv = levels_[L];
        size_t smem = (size_t)lv.max_f * nrhs * sizeof(float);
        mf_fwd_kernel<<<lv.nodes.count, 256, smem, stream_>>>(
            lv.nodes.items, n_, nrhs, d_f_.get(), d_k_.get(), d_own_.get(), d_child0_.get(), d_child1_.get(),
            d_front_off_.get(), d_linv_off_.get(), d_upd_off_.get(), d_map_off_.get(), d_map_.get(), pool_.get(),
            linv_.get(), upd_.get(), d_b, y_.get());
        count_launch();
    }
    for (int L = nlevels_ - 1; L >= 0; --L) {
        Level& lv = levels_[L];
        size_t smem = (size_t)lv.max_f * nrhs * sizeof(float);
        mf_bwd_kernel<<<lv.nodes.count, 256, smem, stream_>>>(lv.nodes.items, n_, nrhs, d_f_.get(), d_k_.get(),
                                                              d_own_.get(), d_front_off_.get(), d_linv_off_.get(),
                                                              d_halo_off_.get(), d_halo_.get(), pool_.get(),
                                                              linv_.get(), D_.get(), y_.get(), d_x);
        count_launch();
    }
    KL_CHECK_LAUNCH();
}

void Multifrontal::stability(double* min_d, int64_t* negatives) {
    const int blocks = 64;
    DevBuf<double> mn(blocks);
    DevBuf<unsigned long long> ng(blocks);
    mf_stability_kernel<<<blocks, 256, 0, stream_>>>(n_, D_.get(), mn.get(), ng.get());
    count_launch();
    KL_CHECK_LAUNCH();
    std::vector<double> hm(blocks);
    std::vector<unsigned long long> hn(blocks);
    mn.download(hm.data(), blocks, stream_);
    ng.download(hn.data(), blocks, stream_);
    KL_CUDA(cudaStreamSynchronize(stream_));
    double m = 1e300;
    unsigned long long s = 0;
    for (int i = 0; i < blocks; ++i) { m = std::min(m, hm[i]); s += hn[i]; }
    *min_d = m;
    *negatives = (int64_t)s;
}

}  // namespace klsa
