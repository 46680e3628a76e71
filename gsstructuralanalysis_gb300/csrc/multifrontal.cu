// multifrontal.cu -- numeric nested-dissection multifrontal LDL^T and triangular solves.
//
// Per level of the elimination tree (leaves first):
//   1. extend-add of the children's Schur complements into the parent fronts (one launch
//      per child slot, so sibling updates never race and the sum order is fixed);
//   2. per 64-column tile step of the pivots: diagonal LDL^T + explicit inverse X = L11^-1 of
//      the unit lower tile (one CTA per front), panel W = A21 X^T and L21 = W D^-1 as a small
//      GEMM (one CTA per 64-row block), trailing lower update A22 -= W L21^T (one CTA per
//      64x64 tile).
// No pivoting (as Eigen's SimplicialLDLT); a zero or non-finite pivot sets the status word.
#include "multifrontal.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <thread>

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

// Extend-add of 8 columns of a child's Schur complement into its parent's front: one warp per
// column, lanes stride over the rows (4 independent read-modify-writes in flight per lane).
constexpr int EA_COLS = 8;
__global__ void __launch_bounds__(256) mf_extend_add_kernel(const int4* __restrict__ items, const int* __restrict__ f,
                                                            const int* __restrict__ k, const int* __restrict__ parent,
                                                            const int64_t* __restrict__ front_off,
                                                            const int64_t* __restrict__ map_off,
                                                            const int* __restrict__ map, float* pool) {
    int4 it = items[blockIdx.x];
    int c = it.x;
    int a = it.y + (threadIdx.x >> 5);
    int lane = threadIdx.x & 31;
    int fc = f[c], kc = k[c], hc = fc - kc;
    if (a >= hc) return;
    int par = parent[c];
    int fp = f[par];
    const int* mp = map + map_off[c];
    const float* scol = pool + front_off[c] + (int64_t)(kc + a) * fc + kc;
    float* dcol = pool + front_off[par] + (int64_t)mp[a] * fp;
    int b = a + lane;
    for (; b + 96 < hc; b += 128) {
        float v0 = scol[b], v1 = scol[b + 32], v2 = scol[b + 64], v3 = scol[b + 96];
        int m0 = mp[b], m1 = mp[b + 32], m2 = mp[b + 64], m3 = mp[b + 96];
        dcol[m0] += v0;
        dcol[m1] += v1;
        dcol[m2] += v2;
        dcol[m3] += v3;
    }
    for (; b < hc; b += 32) dcol[mp[b]] += scol[b];
}

// Diagonal tile (kk <= 64 pivots), 256 threads.  Every entry of the packed lower triangle of the
// 64x64 tile (e = r(r+1)/2 + c) lives in a register of a fixed owner (thread e % 256, slot
// e / 256); rows and columns beyond kk are padded with the identity.
//   LDL^T, right-looking: step j, the owners of column j publish it to shared memory (double
//   buffered), one barrier, then every thread applies -A(r,j) A(c,j) / d_j to its entries with
//   c > j and scales its column-j entries to L(r,j).
//   X = L^-1 (unit lower), same ownership: step j publishes row j of X, rows r > j subtract
//   L(r,j) X(j,:).
// Writes L (strict lower) and D (diagonal) into the front, D into Dvec and X into the tile's slot
// of linv (row-major), which the panel GEMM and the triangular solves use.
constexpr int DIAG_SLOTS = (NB * (NB + 1) / 2 + 255) / 256;
__global__ void __launch_bounds__(256) mf_diag_kernel(const int4* __restrict__ items, int t, const int* __restrict__ f,
                                                      const int* __restrict__ k, const int* __restrict__ own,
                                                      const int64_t* __restrict__ front_off,
                                                      const int64_t* __restrict__ linv_off, float* pool, float* Dvec,
                                                      float* linv, int* status) {
    __shared__ float Ls[NB][NB + 1];
    __shared__ float buf[2][NB];
    __shared__ int bad;
    const int nd = items[blockIdx.x].x;
    const int fN = f[nd], kN = k[nd];
    const int c0 = t * NB;
    const int kk = min(NB, kN - c0);
    float* F = pool + front_off[nd];
    const int tid = threadIdx.x;
    if (tid == 0) bad = 0;
    // stage the tile, column-major walk (coalesced)
    for (int e = tid; e < NB * NB; e += 256) {
        const int c = e / NB, r = e % NB;
        Ls[r][c] = (r < kk && c <= r) ? F[(int64_t)(c0 + c) * fN + c0 + r] : 0.f;
    }
    int rr[DIAG_SLOTS], cc[DIAG_SLOTS];
    float v[DIAG_SLOTS];
#pragma unroll
    for (int q = 0; q < DIAG_SLOTS; ++q) {
        const int e = tid + 256 * q;
        int r = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
        while (r * (r + 1) / 2 > e) --r;
        while ((r + 1) * (r + 2) / 2 <= e) ++r;
        const bool live = e < NB * (NB + 1) / 2;
        rr[q] = live ? r : -1;
        cc[q] = live ? e - r * (r + 1) / 2 : NB;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < DIAG_SLOTS; ++q) {
        const int r = rr[q], c = cc[q];
        v[q] = (r < 0) ? 0.f : (r < kk ? Ls[r][c] : (r == c ? 1.f : 0.f));
    }
    for (int j = 0; j < NB; ++j) {
        float* b = buf[j & 1];
#pragma unroll
        for (int q = 0; q < DIAG_SLOTS; ++q)
            if (cc[q] == j) b[rr[q]] = v[q];
        __syncthreads();
        float d = b[j];
        if (!(fabsf(d) > 0.f) || !isfinite(d)) {
            d = 1.f;
            if (tid == 0) bad = 1;
        }
        const float inv = 1.f / d;
#pragma unroll
        for (int q = 0; q < DIAG_SLOTS; ++q) {
            if (cc[q] > j && cc[q] < NB) v[q] -= b[rr[q]] * inv * b[cc[q]];
            else if (cc[q] == j && rr[q] > j) v[q] *= inv;
        }
    }
    // L and D back to shared memory (the front and the inverse read them from there)
#pragma unroll
    for (int q = 0; q < DIAG_SLOTS; ++q)
        if (rr[q] >= 0) Ls[rr[q]][cc[q]] = v[q];
    __syncthreads();
    for (int e = tid; e < NB * NB; e += 256) {
        const int c = e / NB, r = e % NB;
        if (r < kk && c <= r) F[(int64_t)(c0 + c) * fN + c0 + r] = Ls[r][c];
    }
    if (tid < kk) Dvec[own[nd] + c0 + tid] = Ls[tid][tid];
    // X = L^-1
#pragma unroll
    for (int q = 0; q < DIAG_SLOTS; ++q) v[q] = (rr[q] >= 0 && rr[q] == cc[q]) ? 1.f : 0.f;
    for (int j = 0; j < NB; ++j) {
        float* b = buf[j & 1];
#pragma unroll
        for (int q = 0; q < DIAG_SLOTS; ++q)
            if (rr[q] == j) b[cc[q]] = v[q];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < DIAG_SLOTS; ++q)
            if (rr[q] > j && cc[q] <= j) v[q] -= Ls[rr[q]][j] * b[cc[q]];
    }
    float* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
#pragma unroll
    for (int q = 0; q < DIAG_SLOTS; ++q)
        if (rr[q] >= 0) Li[rr[q] * NB + cc[q]] = rr[q] < kk ? v[q] : 0.f;
    for (int e = tid; e < NB * NB; e += 256)
        if (e % NB > e / NB) Li[e] = 0.f;
    if (tid == 0 && bad && kk > 0) atomicExch(status, 1);
}

// Panel rows [r0, r0 + 64) below the diagonal tile: W = A21 X^T (X = L11^-1 from the diagonal
// kernel), L21 = W D^-1 written in place and W kept for the trailing update.  A 64 x 64 x kk
// product per CTA: thread (tx, ty) owns rows tx + 16 i and columns ty + 16 q.
__global__ void __launch_bounds__(256) mf_panel_kernel(const int4* __restrict__ items, int t, const int* __restrict__ f,
                                                       const int* __restrict__ k, const int64_t* __restrict__ front_off,
                                                       const int64_t* __restrict__ linv_off,
                                                       const int64_t* __restrict__ ws_off, float* pool,
                                                       const float* __restrict__ linv, float* ws) {
    __shared__ float As[NB][NB + 1];   // As[m][rr] = A21(r0 + rr, m)
    __shared__ float Xs[NB][NB + 1];   // Xs[m][jj] = X(jj, m)
    __shared__ float Ds[NB];
    const int4 it = items[blockIdx.x];
    const int nd = it.x, r0 = it.y;
    const int fN = f[nd], kN = k[nd];
    const int c0 = t * NB;
    const int kk = min(NB, kN - c0);
    float* F = pool + front_off[nd];
    const float* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int lt = threadIdx.x & 63, lg = threadIdx.x >> 6;
    {
        float va[16], vx[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int m = lg + 4 * q;
            va[q] = (m < kk && r0 + lt < fN) ? F[(int64_t)(c0 + m) * fN + r0 + lt] : 0.f;
            vx[q] = Li[m * NB + lt];   // X(m, lt): row m of X
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            As[lg + 4 * q][lt] = va[q];
            Xs[lt][lg + 4 * q] = vx[q];
        }
        if (threadIdx.x < NB) Ds[threadIdx.x] = threadIdx.x < kk ? F[(int64_t)(c0 + threadIdx.x) * fN + c0 + threadIdx.x] : 1.f;
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
        for (int q = 0; q < 4; ++q) b[q] = Xs[m][ty + 16 * q];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = fmaf(a[i], b[q], acc[i][q]);
    }
    float* W = ws + ws_off[nd];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int j = ty + 16 * q;
        if (j >= kk) continue;
        const float dinv = 1.f / Ds[j];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int R = r0 + tx + 16 * i;
            if (R < fN) {
                W[(int64_t)j * fN + R] = acc[i][q];
                F[(int64_t)(c0 + j) * fN + R] = acc[i][q] * dinv;
            }
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
    {
        float vw[16], vl[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            int m = lg + 4 * q;
            vw[q] = (m < kk && R0 + lt < fN) ? W[(int64_t)m * fN + R0 + lt] : 0.f;
            vl[q] = (m < kk && C0 + lt < fN) ? F[(int64_t)(c0 + m) * fN + C0 + lt] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            Ws[lg + 4 * q][lt] = vw[q];
            Ls[lg + 4 * q][lt] = vl[q];
        }
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
    float old[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int C = C0 + ty + 16 * q;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int R = R0 + tx + 16 * i;
            old[i][q] = (C < fN && R < fN && R >= C) ? F[(int64_t)C * fN + R] : 0.f;
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int C = C0 + ty + 16 * q;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int R = R0 + tx + 16 * i;
            if (C < fN && R < fN && R >= C) F[(int64_t)C * fN + R] = old[i][q] - acc[i][q];
        }
    }
}

// Forward substitution of one node: children's update vectors, unit-lower solve of the own
// block (inverse diagonal tiles staged in shared memory), update vector of the halo.  Row loops
// are unrolled so that every thread keeps 16 independent loads of L in flight.
constexpr int SOLVE_THREADS = 512;

template <int NR>
__global__ void __launch_bounds__(SOLVE_THREADS) mf_fwd_kernel(const int4* __restrict__ items, int n,
                                                     const int* __restrict__ f, const int* __restrict__ k,
                                                     const int* __restrict__ own, const int* __restrict__ child0,
                                                     const int* __restrict__ child1,
                                                     const int64_t* __restrict__ front_off,
                                                     const int64_t* __restrict__ linv_off,
                                                     const int64_t* __restrict__ upd_off,
                                                     const int64_t* __restrict__ map_off, const int* __restrict__ map,
                                                     const float* __restrict__ pool, const float* __restrict__ linv,
                                                     float* upd, const float* __restrict__ b, float* y) {
    extern __shared__ float rhs[];   // fN * NR
    __shared__ float Ls[NB][NB + 1];
    __shared__ float yt[NR][NB];
    int nd = items[blockIdx.x].x;
    int fN = f[nd], kN = k[nd], hN = fN - kN, o = own[nd];
    const float* F = pool + front_off[nd];
#pragma unroll
    for (int q = 0; q < NR; ++q)
        for (int r = threadIdx.x; r < fN; r += blockDim.x) rhs[r + fN * q] = (r < kN) ? b[o + r + (int64_t)n * q] : 0.f;
    __syncthreads();
    int chs[2] = {child0[nd], child1[nd]};
    for (int s = 0; s < 2; ++s) {
        int c = chs[s];
        if (c >= 0) {
            int hc = f[c] - k[c];
            const int* mp = map + map_off[c];
            const float* u = upd + upd_off[c];
#pragma unroll
            for (int q = 0; q < NR; ++q)
                for (int a = threadIdx.x; a < hc; a += blockDim.x) rhs[mp[a] + fN * q] += u[a + hc * q];
        }
        __syncthreads();
    }
    int ntiles = (kN + NB - 1) / NB;
    for (int t = 0; t < ntiles; ++t) {
        int c0 = t * NB, kk = min(NB, kN - c0);
        const float* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
        {
            float v[NB * NB / SOLVE_THREADS];
#pragma unroll
            for (int q = 0; q < NB * NB / SOLVE_THREADS; ++q) v[q] = Li[threadIdx.x + SOLVE_THREADS * q];
#pragma unroll
            for (int q = 0; q < NB * NB / SOLVE_THREADS; ++q) {
                int e = threadIdx.x + SOLVE_THREADS * q;
                Ls[e / NB][e % NB] = v[q];
            }
        }
        __syncthreads();
        if (threadIdx.x < NB * NR) {
            int j = threadIdx.x % NB, q = threadIdx.x / NB;
            float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;   // Ls is zero above the diagonal
            if (j < kk)
                for (int m = 0; m < kk; m += 4) {
                    a0 += Ls[j][m] * rhs[c0 + m + fN * q];
                    if (m + 1 < kk) a1 += Ls[j][m + 1] * rhs[c0 + m + 1 + fN * q];
                    if (m + 2 < kk) a2 += Ls[j][m + 2] * rhs[c0 + m + 2 + fN * q];
                    if (m + 3 < kk) a3 += Ls[j][m + 3] * rhs[c0 + m + 3 + fN * q];
                }
            yt[q][j] = (a0 + a1) + (a2 + a3);
        }
        __syncthreads();
        if (threadIdx.x < NB * NR) {
            int j = threadIdx.x % NB, q = threadIdx.x / NB;
            if (j < kk) rhs[c0 + j + fN * q] = yt[q][j];
        }
        // rows below the tile: rhs[r] -= L[r, c0:c0+kk] y_t
        for (int r = c0 + kk + threadIdx.x; r < fN; r += blockDim.x) {
            float acc[NR];
#pragma unroll
            for (int q = 0; q < NR; ++q) acc[q] = 0.f;
            const float* col = F + (int64_t)c0 * fN + r;
            int j = 0;
            for (; j + 16 <= kk; j += 16) {
                float l[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) l[u] = col[(int64_t)(j + u) * fN];
#pragma unroll
                for (int u = 0; u < 16; ++u)
#pragma unroll
                    for (int q = 0; q < NR; ++q) acc[q] += l[u] * yt[q][j + u];
            }
            for (; j < kk; ++j) {
                float l = col[(int64_t)j * fN];
#pragma unroll
                for (int q = 0; q < NR; ++q) acc[q] += l * yt[q][j];
            }
#pragma unroll
            for (int q = 0; q < NR; ++q) rhs[r + fN * q] -= acc[q];
        }
        __syncthreads();
    }
    float* u = upd + upd_off[nd];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        for (int r = threadIdx.x; r < kN; r += blockDim.x) y[o + r + (int64_t)n * q] = rhs[r + fN * q];
        for (int a = threadIdx.x; a < hN; a += blockDim.x) u[a + hN * q] = rhs[kN + a + fN * q];
    }
}

// Backward substitution of one node: x_own = L11^-T (D^-1 y_own - L21^T x_halo), tile by tile
// from the last; one warp per column of the tile, lanes stride over the rows below it.
template <int NR>
__global__ void __launch_bounds__(SOLVE_THREADS) mf_bwd_kernel(const int4* __restrict__ items, int n,
                                                     const int* __restrict__ f, const int* __restrict__ k,
                                                     const int* __restrict__ own,
                                                     const int64_t* __restrict__ front_off,
                                                     const int64_t* __restrict__ linv_off,
                                                     const int64_t* __restrict__ halo_off, const int* __restrict__ halo,
                                                     const float* __restrict__ pool, const float* __restrict__ linv,
                                                     const float* __restrict__ Dvec, const float* __restrict__ y,
                                                     float* x) {
    extern __shared__ float xs[];   // fN * NR
    __shared__ float Ls[NB][NB + 1];
    __shared__ float zt[NR][NB];
    int nd = items[blockIdx.x].x;
    int fN = f[nd], kN = k[nd], hN = fN - kN, o = own[nd];
    const float* F = pool + front_off[nd];
    const int* hl = halo + halo_off[nd];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        for (int a = threadIdx.x; a < hN; a += blockDim.x) xs[kN + a + fN * q] = x[hl[a] + (int64_t)n * q];
        for (int r = threadIdx.x; r < kN; r += blockDim.x) xs[r + fN * q] = y[o + r + (int64_t)n * q] / Dvec[o + r];
    }
    __syncthreads();
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    int ntiles = (kN + NB - 1) / NB;
    for (int t = ntiles - 1; t >= 0; --t) {
        int c0 = t * NB, kk = min(NB, kN - c0), c1 = c0 + kk;
        const float* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
        {
            float v[NB * NB / SOLVE_THREADS];
#pragma unroll
            for (int q = 0; q < NB * NB / SOLVE_THREADS; ++q) v[q] = Li[threadIdx.x + SOLVE_THREADS * q];
#pragma unroll
            for (int q = 0; q < NB * NB / SOLVE_THREADS; ++q) {
                int e = threadIdx.x + SOLVE_THREADS * q;
                Ls[e / NB][e % NB] = v[q];
            }
        }
        for (int j = warp; j < kk; j += nwarp) {
            const float* col = F + (int64_t)(c0 + j) * fN;
            float s[NR];
#pragma unroll
            for (int q = 0; q < NR; ++q) s[q] = 0.f;
            int r = c1 + lane;
            for (; r + 96 < fN; r += 128) {
                float l0 = col[r], l1 = col[r + 32], l2 = col[r + 64], l3 = col[r + 96];
#pragma unroll
                for (int q = 0; q < NR; ++q)
                    s[q] += l0 * xs[r + fN * q] + l1 * xs[r + 32 + fN * q] + l2 * xs[r + 64 + fN * q] +
                            l3 * xs[r + 96 + fN * q];
            }
            for (; r < fN; r += 32) {
                float l = col[r];
#pragma unroll
                for (int q = 0; q < NR; ++q) s[q] += l * xs[r + fN * q];
            }
#pragma unroll
            for (int q = 0; q < NR; ++q) {
                float v = s[q];
                for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
                if (lane == 0) zt[q][j] = xs[c0 + j + fN * q] - v;
            }
        }
        __syncthreads();
        if (threadIdx.x < NB * NR) {
            int j = threadIdx.x % NB, q = threadIdx.x / NB;
            if (j < kk) {
                float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;   // Ls[m][j] = 0 for m < j
                for (int m = 0; m < kk; m += 4) {
                    a0 += Ls[m][j] * zt[q][m];
                    if (m + 1 < kk) a1 += Ls[m + 1][j] * zt[q][m + 1];
                    if (m + 2 < kk) a2 += Ls[m + 2][j] * zt[q][m + 2];
                    if (m + 3 < kk) a3 += Ls[m + 3][j] * zt[q][m + 3];
                }
                xs[c0 + j + fN * q] = (a0 + a1) + (a2 + a3);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < NR; ++q)
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
    {
        // rows are independent: split them over the host threads
        const int nt = (int)std::max(1u, std::min(std::thread::hardware_concurrency(), 32u));
        std::vector<std::thread> pool;
        std::vector<int> bad(nt, 0);
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&, t] {
                const int r0 = (int)((int64_t)n_ * t / nt), r1 = (int)((int64_t)n_ * (t + 1) / nt);
                for (int R = r0; R < r1; ++R)
                    for (int e = rowptr[R]; e < rowptr[R + 1]; ++e) {
                        int C = cols[e];
                        if (C > R) continue;
                        int nd = T.node_of[C];
                        int lc = C - T.nodes[nd].own_start;
                        int lr = T.local_index(nd, R);
                        if (lr < 0) { bad[t] = 1; return; }
                        fpos[e] = front_off[nd] + (int64_t)lc * f[nd] + lr;
                    }
            });
        for (auto& th : pool) th.join();
        for (int b : bad)
            if (b) throw std::logic_error("multifrontal: matrix entry outside its front");
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
                for (int a0 = 0; a0 < hc; a0 += EA_COLS) items.push_back(make_int4(c, a0, 0, 0));
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
    // algorithmic traffic and flops per factorisation
    for (int L = 0; L < nlevels_; ++L)
        for (int nd : level_nodes_[L])
            for (int t = 0; t * NB < k[nd]; ++t) {
                double kk = std::min(NB, k[nd] - t * NB);
                double below = f[nd] - t * NB - kk;
                kernel_bytes[0] += 4.0 * kk * kk + 4.0 * NB * NB;      // lower tile in + out, X = L^-1 out
                kernel_flops[0] += 2.0 * kk * kk * kk / 3.0;            // LDL^T + triangular inverse
                kernel_bytes[1] += 4.0 * (3.0 * below * kk + NB * NB);  // A21 in, L21 and W out, X in
                kernel_flops[1] += below * kk * kk;                     // below x kk x kk/2 FMAs
                double ntr = std::ceil(below / NB);
                double tiles = ntr * (ntr + 1) / 2;
                kernel_bytes[2] += tiles * 4.0 * (2.0 * NB * kk + 2.0 * NB * NB);   // W, L tiles in; A tile r/w
                kernel_flops[2] += below * below * kk;                  // lower half of below x below x kk x 2
            }
    for (int i = 0; i < nnodes_; ++i) solve_bytes += 2.0 * 4.0 * ((double)k[i] * f[i] - 0.5 * (double)k[i] * k[i]);
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
    for (int L = 0; L < nlevels_; ++L) {
        for (const Step& st : levels_[L].steps) {
            kernel_launches[0] += st.diag.count > 0;
            kernel_launches[1] += st.panel.count > 0;
            kernel_launches[2] += st.update.count > 0;
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
    int smax = (int)std::max<size_t>(smem, 48 * 1024);
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    KL_CUDA(cudaStreamSynchronize(stream_));
}

namespace {
bool graphs_enabled() {
    static int on = -1;
    if (on < 0) {
        const char* e = std::getenv("KLSA_NO_GRAPHS");
        on = (e && e[0] == '1') ? 0 : 1;
    }
    return on == 1;
}
}  // namespace

// Captures `launches` (a fixed launch sequence on stream_) into a graph once and replays it.
template <class Fn>
void Multifrontal::replay(GraphSlot& slot, const void* key0, const void* key1, Fn&& launches) {
    if (g_timer.enabled || !graphs_enabled()) {
        launches();
        return;
    }
    if (!slot.exec || slot.key0 != key0 || slot.key1 != key1) {
        if (slot.exec) cudaGraphExecDestroy(slot.exec);
        slot.exec = nullptr;
        unsigned long long before = g_launch_count;
        KL_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        try {
            launches();
        } catch (...) {
            cudaGraph_t g;
            cudaStreamEndCapture(stream_, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        cudaGraph_t g;
        KL_CUDA(cudaStreamEndCapture(stream_, &g));
        KL_CUDA(cudaGraphInstantiate(&slot.exec, g, 0));
        cudaGraphDestroy(g);
        slot.kernels = g_launch_count - before;
        g_launch_count = before;
        slot.key0 = key0;
        slot.key1 = key1;
    }
    KL_CUDA(cudaGraphLaunch(slot.exec, stream_));
    count_launch(slot.kernels);
}

Multifrontal::~Multifrontal() {
    for (GraphSlot* s : {&fact_graph_, &solve_graph_[0], &solve_graph_[1], &solve_graph_[2]})
        if (s->exec) cudaGraphExecDestroy(s->exec);
}

void Multifrontal::factorize_async(const float* d_vals) {
    if (!d_vals && nnz_ > 0) throw std::logic_error("multifrontal: no matrix values");
    replay(fact_graph_, d_vals, nullptr, [&] { factorize_launches(d_vals); });
}

void Multifrontal::factorize_launches(const float* d_vals) {
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
                mf_extend_add_kernel<<<lv.ea[s].count, 256, 0, stream_>>>(lv.ea[s].items, d_f_.get(), d_k_.get(),
                                                                          d_parent_.get(), d_front_off_.get(),
                                                                          d_map_off_.get(), d_map_.get(), pool_.get());
                count_launch();
            }
        for (Step& st : lv.steps) {
            if (st.diag.count) {
                cudaEvent_t evk = g_timer.begin(stream_);
                mf_diag_kernel<<<st.diag.count, 256, 0, stream_>>>(st.diag.items, st.t, d_f_.get(), d_k_.get(),
                                                                   d_own_.get(), d_front_off_.get(),
                                                                   d_linv_off_.get(), pool_.get(), D_.get(),
                                                                   linv_.get(), status_.get());
                g_timer.end(stream_, 5, evk);
                count_launch();
            }
            if (st.panel.count) {
                cudaEvent_t evk = g_timer.begin(stream_);
                mf_panel_kernel<<<st.panel.count, 256, 0, stream_>>>(st.panel.items, st.t, d_f_.get(), d_k_.get(),
                                                                     d_front_off_.get(), d_linv_off_.get(),
                                                                     d_ws_off_.get(), pool_.get(), linv_.get(),
                                                                     ws_.get());
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

template <int NR>
void Multifrontal::solve_impl(const float* d_b, float* d_x) {
    for (int L = 0; L < nlevels_; ++L) {
        Level& lv = levels_[L];
        size_t smem = (size_t)lv.max_f * NR * sizeof(float);
        mf_fwd_kernel<NR><<<lv.nodes.count, SOLVE_THREADS, smem, stream_>>>(
            lv.nodes.items, n_, d_f_.get(), d_k_.get(), d_own_.get(), d_child0_.get(), d_child1_.get(),
            d_front_off_.get(), d_linv_off_.get(), d_upd_off_.get(), d_map_off_.get(), d_map_.get(), pool_.get(),
            linv_.get(), upd_.get(), d_b, y_.get());
        count_launch();
    }
    for (int L = nlevels_ - 1; L >= 0; --L) {
        Level& lv = levels_[L];
        size_t smem = (size_t)lv.max_f * NR * sizeof(float);
        mf_bwd_kernel<NR><<<lv.nodes.count, SOLVE_THREADS, smem, stream_>>>(
            lv.nodes.items, n_, d_f_.get(), d_k_.get(), d_own_.get(), d_front_off_.get(), d_linv_off_.get(),
            d_halo_off_.get(), d_halo_.get(), pool_.get(), linv_.get(), D_.get(), y_.get(), d_x);
        count_launch();
    }
    KL_CHECK_LAUNCH();
}

void Multifrontal::enqueue_factorize(const float* d_vals) { factorize_launches(d_vals); }

void Multifrontal::enqueue_solve(const float* d_b, float* d_x) { solve_impl<1>(d_b, d_x); }

void Multifrontal::solve(const float* d_b, float* d_x, int nrhs) {
    switch (nrhs) {
        case 1: replay(solve_graph_[0], d_b, d_x, [&] { solve_impl<1>(d_b, d_x); }); break;
        case 2: replay(solve_graph_[1], d_b, d_x, [&] { solve_impl<2>(d_b, d_x); }); break;
        case 3:
        case 4: {
            // pad to 4 columns: the kernels read/write exactly nrhs columns of ld n
            if (nrhs == 4) { replay(solve_graph_[2], d_b, d_x, [&] { solve_impl<4>(d_b, d_x); }); break; }
            solve_impl<2>(d_b, d_x);
            solve_impl<1>(d_b + 2 * (size_t)n_, d_x + 2 * (size_t)n_);
            break;
        }
        default: throw std::invalid_argument("multifrontal solve: nrhs out of range");
    }
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
