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
#include "tcgen05.cuh"

#include <type_traits>

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <thread>

namespace klsa {

namespace {

constexpr int NB = MF_NB;

template <class T>
__global__ void mf_scatter_kernel(int64_t nnz, const int64_t* __restrict__ fpos, const T* __restrict__ vals,
                                  T* __restrict__ pool) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nnz) {
        int64_t p = fpos[i];
        if (p >= 0) pool[p] = vals[i];
    }
}

// Extend-add of 8 columns of a child's Schur complement into its parent's front: one warp per
// column, lanes stride over the rows (4 independent read-modify-writes in flight per lane).
constexpr int EA_COLS = 8;
template <class T>
__global__ void __launch_bounds__(256) mf_extend_add_kernel(const int4* __restrict__ items, const int* __restrict__ f,
                                                            const int* __restrict__ k, const int* __restrict__ parent,
                                                            const int64_t* __restrict__ front_off,
                                                            const int64_t* __restrict__ map_off,
                                                            const int* __restrict__ map, T* pool) {
    int4 it = items[blockIdx.x];
    int c = it.x;
    int a = it.y + (threadIdx.x >> 5);
    int lane = threadIdx.x & 31;
    int fc = f[c], kc = k[c], hc = fc - kc;
    if (a >= hc) return;
    int par = parent[c];
    int fp = f[par];
    const int* mp = map + map_off[c];
    const T* scol = pool + front_off[c] + (int64_t)(kc + a) * fc + kc;
    T* dcol = pool + front_off[par] + (int64_t)mp[a] * fp;
    int b = a + lane;
    for (; b + 96 < hc; b += 128) {
        T v0 = scol[b], v1 = scol[b + 32], v2 = scol[b + 64], v3 = scol[b + 96];
        int m0 = mp[b], m1 = mp[b + 32], m2 = mp[b + 64], m3 = mp[b + 96];
        dcol[m0] += v0;
        dcol[m1] += v1;
        dcol[m2] += v2;
        dcol[m3] += v3;
    }
    for (; b < hc; b += 32) dcol[mp[b]] += scol[b];
}

// Diagonal tile (kk <= 64 pivots), 288 threads.  Thread t owns one row r of the tile and the 8
// columns [8q, 8q + 8) of it that lie on or below the diagonal (q = 0..7, rows r >= 8q: 64 + 56 +
// ... + 8 = 288 owners), both of A (becoming L and D) and of X = L^-1 (unit lower); rows and
// columns beyond kk are padded with the identity.  Step j (one barrier): the owners of column j
// publish A(:, j), the owner of the pivot its reciprocal, the owners of row j of X publish
// X(j, :).  Then every thread updates its 8 entries:
//   A(r, c) -= L(r, j) A(c, j) for c > j,   A(r, j) = L(r, j) = A(r, j) / d_j,
//   X(r, c) -= L(r, j) X(j, c) for c <= j < r.
// A thread reads one value of column j for its row and two 16-byte words of the column / row
// buffers that its whole column group shares, so the shared-memory traffic per step stays small.
// Writes L (strict lower) and D into the front, D into Dvec and X into the tile's slot of linv
// (row-major), which the panel GEMM and the triangular solves use.
constexpr int DIAG_THREADS = 288;

// 1/d from the fast intrinsic quotient refined by Newton's iteration r <- r (2 - d r), with the
// exact quotient outside the range where the intrinsic is accurate.
__device__ __forceinline__ float pivot_recip(float d) {
    const float ad = fabsf(d);
    if (!(ad > 1e-30f && ad < 1e30f)) return 1.0f / d;
    const float r = __fdividef(1.0f, d);
    return r * (2.0f - d * r);
}
__device__ __forceinline__ double pivot_recip(double d) {
    const double ad = fabs(d);
    if (!(ad > 1e-30 && ad < 1e30)) return 1.0 / d;
    double r = (double)__fdividef(1.0f, (float)d);
    r = r * (2.0 - d * r);
    return r * (2.0 - d * r);
}

template <class T>
__device__ __forceinline__ T sel8(const T (&v)[8], int k) {
    T r = v[0];
#pragma unroll
    for (int q = 1; q < 8; ++q) r = (k == q) ? v[q] : r;
    return r;
}

template <class T>
__global__ void __launch_bounds__(DIAG_THREADS) mf_diag_kernel(const int4* __restrict__ items, int t,
                                                               const int* __restrict__ f, const int* __restrict__ k,
                                                               const int* __restrict__ own,
                                                               const int64_t* __restrict__ front_off,
                                                               const int64_t* __restrict__ linv_off, T* pool, T* Dvec,
                                                               T* linv, int* status) {
    // published per pivot pair (j, j+1), double-buffered by pair parity: columns j and j+1 of A
    // (rows >= j) and rows j, j+1 of X
    __shared__ __align__(16) T col0s[2][NB];
    __shared__ __align__(16) T col1s[2][NB];
    __shared__ __align__(16) T xr0s[2][NB];
    __shared__ __align__(16) T xr1s[2][NB];
    __shared__ int bad;
    const int nd = items[blockIdx.x].x;
    const int fN = f[nd], kN = k[nd];
    const int c0 = t * NB;
    const int kk = min(NB, kN - c0);
    T* F = pool + front_off[nd];
    const int tid = threadIdx.x;
    // owner map: column group q and row r (rows 8q..63 of group q)
    int q = 0, base = 0;
    while (q < 7 && tid >= base + (NB - 8 * q)) {
        base += NB - 8 * q;
        ++q;
    }
    const int r = 8 * q + (tid - base);
    const int cb = 8 * q;
    T a[8], x[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int c = cb + e;
        a[e] = (c > r) ? T(0) : (r < kk ? F[(int64_t)(c0 + c) * fN + c0 + r] : (r == c ? T(1) : T(0)));
        x[e] = (r == c) ? T(1) : T(0);
    }
    if (tid == 0) bad = 0;
    // pivot pairs, one barrier each (the pair two steps back used the same buffers, and every
    // thread has passed the previous pair's barrier since reading them); pivots beyond kk are the
    // identity padding (an odd kk pairs its last pivot with a padding pivot)
    for (int jq = 0; jq * 8 < kk; ++jq) {
#pragma unroll
        for (int jj = 0; jj < 8; jj += 2) {
            const int j = jq * 8 + jj;
            if (j < kk) {
                const int pb = (jj >> 1) & 1;
                T* col0 = col0s[pb];
                T* col1 = col1s[pb];
                T* xr0 = xr0s[pb];
                T* xr1 = xr1s[pb];
                if (jq == q && r >= j) {
                    col0[r] = a[jj];
                    col1[r] = a[jj + 1];
                }
                if (r == j) {
#pragma unroll
                    for (int e = 0; e < 8; ++e) xr0[cb + e] = x[e];
                }
                if (r == j + 1) {
#pragma unroll
                    for (int e = 0; e < 8; ++e) xr1[cb + e] = x[e];
                }
                __syncthreads();
                // the 2x2 pivot block, rebuilt by every thread
                T d0 = col0[j];
                const T e10 = col0[j + 1], f11 = col1[j + 1];
                if (!(fabs(d0) > T(0)) || !isfinite(d0)) {
                    if (tid == 0) bad = 1;
                    d0 = T(1);
                }
                const T inv0 = pivot_recip(d0);
                const T l10 = e10 * inv0;
                T d1 = f11 - l10 * e10;
                if (!(fabs(d1) > T(0)) || !isfinite(d1)) {
                    if (tid == 0 && j + 1 < kk) bad = 1;
                    d1 = T(1);
                }
                const T inv1 = pivot_recip(d1);
                // own row: L(r, j), column j+1 after the column-j update, L(r, j+1)
                const T lr0 = col0[r] * inv0;
                const T ar1 = col1[r] - lr0 * e10;
                const T lr1 = ar1 * inv1;
                const T g = inv0 * e10;
                if (q > jq) {
                    // every column right of the pair: rank-2 update only
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const T cv0 = col0[cb + e], cv1 = col1[cb + e];
                        const T an = a[e] - lr0 * cv0 - lr1 * (cv1 - cv0 * g);
                        a[e] = (cb + e <= r) ? an : a[e];
                    }
                } else if (q < jq) {
                    // every column left of the pair: only X changes, in the rows below it
                    if (r > j) {
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            const T xv0 = xr0[cb + e], xv1 = xr1[cb + e];
                            const T xn2 = x[e] - lr0 * xv0 - lr1 * (xv1 - l10 * xv0);
                            const T xn1 = x[e] - l10 * xv0;
                            x[e] = (r > j + 1) ? xn2 : xn1;
                        }
                    }
                } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int c = cb + e;
                        const T cv0 = col0[c], cv1 = col1[c], xv0 = xr0[c], xv1 = xr1[c];
                        // A: rank-2 update of c > j+1, columns j and j+1 become L, the pivot
                        // (j+1, j+1) d1
                        const T an = a[e] - lr0 * cv0 - lr1 * (cv1 - cv0 * g);
                        T av = a[e];
                        if (c > j + 1 && c <= r) av = an;
                        else if (c == j && r > j) av = lr0;
                        else if (c == j + 1 && r > j + 1) av = lr1;
                        else if (c == j + 1 && r == j + 1) av = d1;
                        a[e] = av;
                        // X: rows below the pair take both steps, row j+1 the first
                        const T xn2 = x[e] - lr0 * xv0 - lr1 * (xv1 - l10 * xv0);
                        const T xn1 = x[e] - l10 * xv0;
                        T xv = x[e];
                        if (c <= j + 1 && r > j + 1) xv = xn2;
                        else if (c <= j && r == j + 1) xv = xn1;
                        x[e] = xv;
                    }
                }
            }
        }
    }
    T* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int c = cb + e;
        if (c <= r) {
            if (r < kk) F[(int64_t)(c0 + c) * fN + c0 + r] = a[e];
            Li[r * NB + c] = r < kk ? x[e] : T(0);
        }
    }
    if (r >= cb && r < cb + 8 && r < kk) Dvec[own[nd] + c0 + r] = sel8(a, r - cb);
    for (int e = tid; e < NB * NB; e += DIAG_THREADS)
        if (e % NB > e / NB) Li[e] = T(0);
    __syncthreads();
    if (tid == 0 && bad) atomicExch(status, 1);
}

// Four consecutive shared-memory values (16-byte aligned) in one or two vector loads.
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
    const float4 x = *reinterpret_cast<const float4*>(p);
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
    const double2 x = *reinterpret_cast<const double2*>(p);
    const double2 y = *reinterpret_cast<const double2*>(p + 2);
    v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
}

// Staged 64-wide tiles use rows padded to NBP = 68 elements, keeping the vectors aligned.
constexpr int NBP = NB + 4;

// Panel rows [r0, r0 + 64) below the diagonal tile: W = A21 X^T (X = L11^-1 from the diagonal
// kernel), L21 = W D^-1 written in place and W kept for the trailing update.  A 64 x 64 x kk
// product per CTA: thread (tx, ty) owns rows tx + 16 i and columns ty + 16 q.
template <class T>
__global__ void __launch_bounds__(256) mf_panel_kernel(const int4* __restrict__ items, int t, const int* __restrict__ f,
                                                       const int* __restrict__ k, const int64_t* __restrict__ front_off,
                                                       const int64_t* __restrict__ linv_off,
                                                       const int64_t* __restrict__ ws_off, T* pool,
                                                       const T* __restrict__ linv, T* ws) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T(*As)[NB + 1] = reinterpret_cast<T(*)[NB + 1]>(smem_raw);              // As[m][rr] = A21(r0 + rr, m)
    T(*Xs)[NB + 1] = reinterpret_cast<T(*)[NB + 1]>(smem_raw + sizeof(T) * NB * (NB + 1));   // Xs[m][jj] = X(jj, m)
    T* Ds = reinterpret_cast<T*>(smem_raw + 2 * sizeof(T) * NB * (NB + 1));
    const int4 it = items[blockIdx.x];
    const int nd = it.x, r0 = it.y;
    const int fN = f[nd], kN = k[nd];
    const int c0 = t * NB;
    const int kk = min(NB, kN - c0);
    T* F = pool + front_off[nd];
    const T* Li = linv + linv_off[nd] + (int64_t)t * NB * NB;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int lt = threadIdx.x & 63, lg = threadIdx.x >> 6;
    {
        T va[16], vx[16];
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
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[i][q] = 0.f;
    for (int m = 0; m < kk; ++m) {
        T a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[m][tx + 16 * i];
#pragma unroll
        for (int q = 0; q < 4; ++q) b[q] = Xs[m][ty + 16 * q];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = fma(a[i], b[q], acc[i][q]);
    }
    T* W = ws + ws_off[nd];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int j = ty + 16 * q;
        if (j >= kk) continue;
        const T dinv = 1.f / Ds[j];
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

// Trailing update of one 64x64 lower tile: A[R, C] -= W[R, :] L[C, :]^T.  Thread (tx, ty) owns
// rows 4tx..4tx+3 and columns 4ty..4ty+3; per k step two 16-byte shared loads feed 16 FMAs.
template <class T>
__global__ void __launch_bounds__(256) mf_update_kernel(const int4* __restrict__ items, int t, const int* __restrict__ f,
                                                        const int* __restrict__ k, const int64_t* __restrict__ front_off,
                                                        const int64_t* __restrict__ ws_off, T* pool,
                                                        const T* __restrict__ ws) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T(*Ws)[NBP] = reinterpret_cast<T(*)[NBP]>(smem_raw);                          // Ws[m][rr] = W[R0+rr][m]
    T(*Ls)[NBP] = reinterpret_cast<T(*)[NBP]>(smem_raw + sizeof(T) * NB * NBP);   // Ls[m][cc] = L[C0+cc][c0+m]
    const int4 it = items[blockIdx.x];
    const int nd = it.x;
    const int fN = f[nd], kN = k[nd];
    const int c0 = t * NB;
    const int kk = min(NB, kN - c0);
    const int c1 = c0 + kk;
    const int R0 = c1 + it.y * NB, C0 = c1 + it.z * NB;
    T* F = pool + front_off[nd];
    const T* W = ws + ws_off[nd];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int lt = threadIdx.x & 63, lg = threadIdx.x >> 6;
    {
        T vw[16], vl[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int m = lg + 4 * q;
            vw[q] = (m < kk && R0 + lt < fN) ? W[(int64_t)m * fN + R0 + lt] : T(0);
            vl[q] = (m < kk && C0 + lt < fN) ? F[(int64_t)(c0 + m) * fN + C0 + lt] : T(0);
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            Ws[lg + 4 * q][lt] = vw[q];
            Ls[lg + 4 * q][lt] = vl[q];
        }
    }
    __syncthreads();
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
#pragma unroll 4
    for (int m = 0; m < kk; ++m) {
        T a[4], b[4];
        ld4(&Ws[m][4 * tx], a);
        ld4(&Ls[m][4 * ty], b);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    T old[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int C = C0 + 4 * ty + j;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int R = R0 + 4 * tx + i;
            old[i][j] = (C < fN && R < fN && R >= C) ? F[(int64_t)C * fN + R] : T(0);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int C = C0 + 4 * ty + j;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int R = R0 + 4 * tx + i;
            if (C < fN && R < fN && R >= C) F[(int64_t)C * fN + R] = old[i][j] - acc[i][j];
        }
    }
}

// The same trailing update on the 5th-generation tensor cores (FP32 fronts).  One CTA of 128
// threads per 64 x 64 lower tile: the W and L blocks (K = kk <= 64, zero-padded to a multiple
// of 8) are split into TF32 high and low parts, hi = tf32(x) and lo = x - hi, and staged
// K-major in shared memory; one thread issues D = Wh Lh^T + Wh Ll^T + Wl Lh^T as tcgen05
// kind::tf32 MMAs (M = 128, of which rows 0..63 are the tile; N = 64, K = 8 each) into a
// 64-column FP32 accumulator in tensor memory, committed to an mbarrier.  Three-term TF32
// splitting keeps the product at FP32 accuracy (the dropped lo*lo term is below 2^-22
// relative).  Warps 0 and 1 read their 32 accumulator lanes each and subtract them from the
// front.  The wait for the MMAs is bounded: on expiry the status flag is raised, the tile is
// left unchanged and the tensor memory is still released.
constexpr int TC_THREADS = 128;
constexpr int TC_TILE_BYTES = NB * NB * 4;   // one 64 x 64 FP32 operand tile
constexpr size_t TC_SMEM = 4 * (size_t)TC_TILE_BYTES;

__global__ void __launch_bounds__(TC_THREADS) mf_update_tc_kernel(const int4* __restrict__ items, int t,
                                                                  const int* __restrict__ f, const int* __restrict__ k,
                                                                  const int64_t* __restrict__ front_off,
                                                                  const int64_t* __restrict__ ws_off, float* pool,
                                                                  const float* __restrict__ ws, int* status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tholder;
    // [Wh | Wl | Lh | Ll]; the M = 128 MMA reads 128 rows of Wh and Wl, the second half of which
    // lies in the next operand tile and lands in accumulator rows 64..127, which are not used
    float* Wh = reinterpret_cast<float*>(smem_raw);
    float* Wl = Wh + NB * NB;
    float* Lh = Wl + NB * NB;
    float* Ll = Lh + NB * NB;
    const int4 it = items[blockIdx.x];
    const int nd = it.x;
    const int fN = f[nd], kN = k[nd];
    const int c0 = t * NB;
    const int kk = min(NB, kN - c0);
    const int k8 = (kk + 7) & ~7;
    const int R0 = c0 + kk + it.y * NB, C0 = c0 + kk + it.z * NB;
    float* F = pool + front_off[nd];
    const float* W = ws + ws_off[nd];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tc::tmem_alloc(&tholder, 64);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    {
        // every load in flight first (consecutive threads: consecutive rows of one column), then
        // the split and the K-major stores
        constexpr int PER = NB * NB / TC_THREADS;
        float vw[PER], vl[PER];
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int e = tid + TC_THREADS * q, r = e % NB, m = e / NB;
            vw[q] = (m < kk && R0 + r < fN) ? W[(int64_t)m * fN + R0 + r] : 0.f;
            vl[q] = (m < kk && C0 + r < fN) ? F[(int64_t)(c0 + m) * fN + C0 + r] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int e = tid + TC_THREADS * q, r = e % NB, m = e / NB;
            if (m < k8) {
                const float wh = tc::to_tf32(vw[q]), lh = tc::to_tf32(vl[q]);
                const uint32_t o = tc::kmajor_offset(r, m, NB / 4) >> 2;
                Wh[o] = wh;
                Wl[o] = vw[q] - wh;
                Lh[o] = lh;
                Ll[o] = vl[q] - lh;
            }
        }
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tholder;
    if (tid == 0) {
        constexpr uint32_t LBO = 128, SBO = 128 * (NB / 4);
        const uint32_t idesc = tc::idesc_tf32(128, 64);
        const uint32_t wh = tc::smem_u32(Wh), wl = tc::smem_u32(Wl), lh = tc::smem_u32(Lh), ll = tc::smem_u32(Ll);
        for (int s8 = 0; s8 < k8 / 8; ++s8) {
            const uint32_t o = 256u * s8;   // two core matrices along K per MMA
            const uint64_t dwh = tc::smem_desc_kmajor(wh + o, LBO, SBO), dwl = tc::smem_desc_kmajor(wl + o, LBO, SBO);
            const uint64_t dlh = tc::smem_desc_kmajor(lh + o, LBO, SBO), dll = tc::smem_desc_kmajor(ll + o, LBO, SBO);
            tc::mma_tf32(taddr, dwh, dlh, idesc, s8 > 0);
            tc::mma_tf32(taddr, dwh, dll, idesc, true);
            tc::mma_tf32(taddr, dwl, dlh, idesc, true);
        }
        tc::commit(&mbar);
    }
    bool ok = tc::mbar_wait(&mbar, 0, 1u << 20);
    if (!ok) ok = tc::mbar_wait(&mbar, 0, 1u << 20);
    tc::fence_after_sync();
    if (ok && warp < 2 && k8 > 0) {
        const int r = 32 * warp + lane, R = R0 + r;
#pragma unroll
        for (int cc = 0; cc < NB; cc += 16) {
            float v[16];
            tc::ld_32x32b_x16(taddr + (static_cast<uint32_t>(32 * warp) << 16) + cc, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int C = C0 + cc + i;
                if (C < fN && R < fN && R >= C) F[(int64_t)C * fN + R] -= v[i];
            }
        }
    }
    if (!ok && tid == 0) atomicExch(status, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(taddr, 64);
}

// ---- node inverses X = L11^-1 (k x k, row-major, lower) for the triangular solves -------------
// Diagonal blocks: copies of the tile inverses written by the diagonal kernel.
template <class T>
__global__ void __launch_bounds__(256) mf_xdiag_kernel(const int4* __restrict__ items, const int* __restrict__ k,
                                                       const int64_t* __restrict__ linv_off,
                                                       const int64_t* __restrict__ xinv_off,
                                                       const T* __restrict__ linv, T* __restrict__ xinv) {
    const int4 it = items[blockIdx.x];
    const int nd = it.x, bi = it.y, kN = k[nd];
    const int c0 = bi * NB, kk = min(NB, kN - c0);
    const T* Li = linv + linv_off[nd] + (int64_t)bi * NB * NB;
    T* X = xinv + xinv_off[nd];
    for (int e = threadIdx.x; e < NB * NB; e += 256) {
        const int r = e / NB, c = e % NB;
        if (r < kk && c < kk) X[(int64_t)(c0 + r) * kN + c0 + c] = Li[e];
    }
}

// Block row bi of X, block column bj < bi: X(bi, bj) = -X(bi, bi) sum_{m=bj}^{bi-1} L(bi, m) X(m, bj).
// One CTA per output tile; thread (tx, ty) owns rows tx + 16 i and columns ty + 16 q.
template <class T>
__global__ void __launch_bounds__(256) mf_xoff_kernel(const int4* __restrict__ items, const int* __restrict__ f,
                                                      const int* __restrict__ k, const int64_t* __restrict__ front_off,
                                                      const int64_t* __restrict__ linv_off,
                                                      const int64_t* __restrict__ xinv_off, const T* __restrict__ pool,
                                                      const T* __restrict__ linv, T* __restrict__ xinv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T(*As)[NB + 1] = reinterpret_cast<T(*)[NB + 1]>(smem_raw);                               // As[q][r] = L(bi, m)(r, q)
    T(*Bs)[NB + 1] = reinterpret_cast<T(*)[NB + 1]>(smem_raw + sizeof(T) * NB * (NB + 1));   // Bs[q][c] = X(m, bj)(q, c)
    const int4 it = items[blockIdx.x];
    const int nd = it.x, bi = it.y, bj = it.z;
    const int fN = f[nd], kN = k[nd];
    const int ri = bi * NB, kki = min(NB, kN - ri), cj = bj * NB;
    const T* F = pool + front_off[nd];
    T* X = xinv + xinv_off[nd];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int lt = threadIdx.x & 63, lg = threadIdx.x >> 6;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[i][q] = T(0);
    for (int bm = bj; bm < bi; ++bm) {
        const int cm = bm * NB;
        __syncthreads();
        {
            T va[16], vb[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int qq = lg + 4 * q;
                va[q] = lt < kki ? F[(int64_t)(cm + qq) * fN + ri + lt] : T(0);   // L(ri + lt, cm + qq)
                vb[q] = X[(int64_t)(cm + qq) * kN + cj + lt];                   // X(cm + qq, cj + lt)
            }
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                As[lg + 4 * q][lt] = va[q];
                Bs[lg + 4 * q][lt] = vb[q];
            }
        }
        __syncthreads();
        for (int q = 0; q < NB; ++q) {
            T av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[q][tx + 16 * i];
#pragma unroll
            for (int c = 0; c < 4; ++c) bv[c] = Bs[q][ty + 16 * c];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[i][c] = fma(av[i], bv[c], acc[i][c]);
        }
    }
    // S -> shared (Bs[r][c]), X(bi, bi) -> shared (As[r][q] = Xii(r, q)), out = -Xii S
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 4; ++c) Bs[tx + 16 * i][ty + 16 * c] = acc[i][c];
    const T* Li = linv + linv_off[nd] + (int64_t)bi * NB * NB;
    for (int e = threadIdx.x; e < NB * NB; e += 256) As[e / NB][e % NB] = Li[e];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[i][c] = T(0);
    for (int q = 0; q < NB; ++q) {
        T av[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) av[i] = As[tx + 16 * i][q];
#pragma unroll
        for (int c = 0; c < 4; ++c) bv[c] = Bs[q][ty + 16 * c];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[i][c] = fma(av[i], bv[c], acc[i][c]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = tx + 16 * i;
        if (r < kki)
#pragma unroll
            for (int c = 0; c < 4; ++c) X[(int64_t)(ri + r) * kN + cj + ty + 16 * c] = -acc[i][c];
    }
}

// ---- triangular solves, five launches per level, many CTAs per front ---------------------------
// Forward, leaves first: (1) gather b and the children's update vectors into the own part (y) and
// the halo part (upd) of every node; (2) z_own = X r_own (row blocks); (3) u = r_halo - L21 z_own
// (halo row blocks).  Backward, root first: (4) w = D^-1 z_own - L21^T x_halo (own column
// blocks); (5) x_own = X^T w (own column blocks).  Vectors: n x NR, column stride n.
constexpr int SOLVE_THREADS = 256;

template <class T, int NR>
__global__ void __launch_bounds__(SOLVE_THREADS) mf_fwd_gather_kernel(
    const int4* __restrict__ items, int n, const int* __restrict__ f, const int* __restrict__ k,
    const int* __restrict__ own, const int* __restrict__ child0, const int* __restrict__ child1,
    const int64_t* __restrict__ upd_off, const int64_t* __restrict__ map_off, const int* __restrict__ map,
    const T* __restrict__ b, T* __restrict__ y, T* upd) {
    const int nd = items[blockIdx.x].x;
    const int kN = k[nd], hN = f[nd] - kN, o = own[nd];
    T* u = upd + upd_off[nd];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        for (int r = threadIdx.x; r < kN; r += blockDim.x) y[o + r + (int64_t)n * q] = b[o + r + (int64_t)n * q];
        for (int a = threadIdx.x; a < hN; a += blockDim.x) u[a + hN * q] = T(0);
    }
    const int chs[2] = {child0[nd], child1[nd]};
    for (int s = 0; s < 2; ++s) {
        __syncthreads();
        const int c = chs[s];
        if (c < 0) continue;
        const int hc = f[c] - k[c];
        const int* mp = map + map_off[c];
        const T* uc = upd + upd_off[c];
#pragma unroll
        for (int q = 0; q < NR; ++q)
            for (int a = threadIdx.x; a < hc; a += blockDim.x) {
                const int pos = mp[a];
                if (pos < kN) y[o + pos + (int64_t)n * q] += uc[a + hc * q];
                else u[pos - kN + hN * q] += uc[a + hc * q];
            }
    }
}

// z_own(i) = sum_{m <= i} X(i, m) y_own(m); warp w handles rows rb*64 + w*8 .. +8, lanes over m.
template <class T, int NR>
__global__ void __launch_bounds__(SOLVE_THREADS) mf_fwd_own_kernel(
    const int4* __restrict__ items, int n, const int* __restrict__ k, const int* __restrict__ own,
    const int64_t* __restrict__ xinv_off, const T* __restrict__ xinv, const T* __restrict__ y, T* __restrict__ z) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* ys = reinterpret_cast<T*>(smem_raw);   // kN * NR
    const int4 it = items[blockIdx.x];
    const int nd = it.x, rb = it.y;
    const int kN = k[nd], o = own[nd];
    const int r1 = min(kN, (rb + 1) * NB);
#pragma unroll
    for (int q = 0; q < NR; ++q)
        for (int m = threadIdx.x; m < r1; m += blockDim.x) ys[m + kN * q] = y[o + m + (int64_t)n * q];
    __syncthreads();
    const T* X = xinv + xinv_off[nd];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int rr = 0; rr < 8; ++rr) {
        const int i = rb * NB + warp * 8 + rr;
        if (i >= kN) break;
        const T* xr = X + (int64_t)i * kN;
        T s[NR];
#pragma unroll
        for (int q = 0; q < NR; ++q) s[q] = T(0);
        for (int m = lane; m <= i; m += 32) {
            const T xv = xr[m];
#pragma unroll
            for (int q = 0; q < NR; ++q) s[q] += xv * ys[m + kN * q];
        }
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            T v = s[q];
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) z[o + i + (int64_t)n * q] = v;
        }
    }
}

// u(a) -= sum_j L21(a, j) z_own(j) for halo rows a of block ab; thread (al, g): row al, j = g mod 4.
template <class T, int NR>
__global__ void __launch_bounds__(SOLVE_THREADS) mf_fwd_halo_kernel(
    const int4* __restrict__ items, int n, const int* __restrict__ f, const int* __restrict__ k,
    const int* __restrict__ own, const int64_t* __restrict__ front_off, const int64_t* __restrict__ upd_off,
    const T* __restrict__ pool, const T* __restrict__ z, T* upd) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* zs = reinterpret_cast<T*>(smem_raw);                                  // kN * NR
    __shared__ T part[4][NR][NB];
    const int4 it = items[blockIdx.x];
    const int nd = it.x, ab = it.y;
    const int fN = f[nd], kN = k[nd], hN = fN - kN, o = own[nd];
#pragma unroll
    for (int q = 0; q < NR; ++q)
        for (int m = threadIdx.x; m < kN; m += blockDim.x) zs[m + kN * q] = z[o + m + (int64_t)n * q];
    __syncthreads();
    const T* F = pool + front_off[nd];
    const int al = threadIdx.x & 63, g = threadIdx.x >> 6;
    const int a = ab * NB + al;
    T s[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) s[q] = T(0);
    if (a < hN) {
        const T* col = F + kN + a;
        int j = g;
        for (; j + 12 < kN; j += 16) {
            const T l0 = col[(int64_t)j * fN], l1 = col[(int64_t)(j + 4) * fN];
            const T l2 = col[(int64_t)(j + 8) * fN], l3 = col[(int64_t)(j + 12) * fN];
#pragma unroll
            for (int q = 0; q < NR; ++q)
                s[q] += l0 * zs[j + kN * q] + l1 * zs[j + 4 + kN * q] + l2 * zs[j + 8 + kN * q] +
                        l3 * zs[j + 12 + kN * q];
        }
        for (; j < kN; j += 4) {
            const T l = col[(int64_t)j * fN];
#pragma unroll
            for (int q = 0; q < NR; ++q) s[q] += l * zs[j + kN * q];
        }
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) part[g][q][al] = s[q];
    __syncthreads();
    if (g == 0 && a < hN) {
        T* u = upd + upd_off[nd];
#pragma unroll
        for (int q = 0; q < NR; ++q)
            u[a + hN * q] -= (part[0][q][al] + part[1][q][al]) + (part[2][q][al] + part[3][q][al]);
    }
}

// w(j) = z(j) / D(j) - sum_a L21(a, j) x(halo a) for own columns j of block jb; warp per column.
template <class T, int NR>
__global__ void __launch_bounds__(SOLVE_THREADS) mf_bwd_z_kernel(
    const int4* __restrict__ items, int n, const int* __restrict__ f, const int* __restrict__ k,
    const int* __restrict__ own, const int64_t* __restrict__ front_off, const int64_t* __restrict__ halo_off,
    const int* __restrict__ halo, const T* __restrict__ pool, const T* __restrict__ Dvec, const T* __restrict__ z,
    const T* __restrict__ x, T* __restrict__ w) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* xs = reinterpret_cast<T*>(smem_raw);   // hN * NR
    const int4 it = items[blockIdx.x];
    const int nd = it.x, jb = it.y;
    const int fN = f[nd], kN = k[nd], hN = fN - kN, o = own[nd];
    const int* hl = halo + halo_off[nd];
#pragma unroll
    for (int q = 0; q < NR; ++q)
        for (int a = threadIdx.x; a < hN; a += blockDim.x) xs[a + hN * q] = x[hl[a] + (int64_t)n * q];
    __syncthreads();
    const T* F = pool + front_off[nd];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int jj = 0; jj < 8; ++jj) {
        const int j = jb * NB + warp * 8 + jj;
        if (j >= kN) break;
        const T* col = F + (int64_t)j * fN + kN;
        T s[NR];
#pragma unroll
        for (int q = 0; q < NR; ++q) s[q] = T(0);
        for (int a = lane; a < hN; a += 32) {
            const T l = col[a];
#pragma unroll
            for (int q = 0; q < NR; ++q) s[q] += l * xs[a + hN * q];
        }
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            T v = s[q];
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) w[o + j + (int64_t)n * q] = z[o + j + (int64_t)n * q] / Dvec[o + j] - v;
        }
    }
}

// x_own(j) = sum_{i >= j} X(i, j) w(i) for own columns j of block jb; thread (jl, g): column jl,
// rows i = g mod 4 (row-major X: a row segment of 64 columns per load).
template <class T, int NR>
__global__ void __launch_bounds__(SOLVE_THREADS) mf_bwd_own_kernel(
    const int4* __restrict__ items, int n, const int* __restrict__ k, const int* __restrict__ own,
    const int64_t* __restrict__ xinv_off, const T* __restrict__ xinv, const T* __restrict__ w, T* __restrict__ x) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* ws = reinterpret_cast<T*>(smem_raw);   // kN * NR
    __shared__ T part[4][NR][NB];
    const int4 it = items[blockIdx.x];
    const int nd = it.x, jb = it.y;
    const int kN = k[nd], o = own[nd];
    const int j0 = jb * NB;
#pragma unroll
    for (int q = 0; q < NR; ++q)
        for (int i = j0 + threadIdx.x; i < kN; i += blockDim.x) ws[i + kN * q] = w[o + i + (int64_t)n * q];
    __syncthreads();
    const T* X = xinv + xinv_off[nd];
    const int jl = threadIdx.x & 63, g = threadIdx.x >> 6;
    const int j = j0 + jl;
    T s[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) s[q] = T(0);
    if (j < kN)
        for (int i = j0 + g; i < kN; i += 4) {
            const T xv = (i >= j) ? X[(int64_t)i * kN + j] : T(0);
#pragma unroll
            for (int q = 0; q < NR; ++q) s[q] += xv * ws[i + kN * q];
        }
#pragma unroll
    for (int q = 0; q < NR; ++q) part[g][q][jl] = s[q];
    __syncthreads();
    if (g == 0 && j < kN)
#pragma unroll
        for (int q = 0; q < NR; ++q)
            x[o + j + (int64_t)n * q] = (part[0][q][jl] + part[1][q][jl]) + (part[2][q][jl] + part[3][q][jl]);
}

// ---- triangular solves in one persistent cooperative launch --------------------------------------
// The products of the five-launch solve above, cut into 64 x 64 tiles of X = L11^-1 and L21 so
// that every phase offers hundreds to thousands of independent tiles: one tile is one round of
// 16 independent loads per thread, and its partial mat-vec is added atomically into the target
// vector.  One grid walks all levels with a grid-wide barrier between phases:
//   forward (leaves first), per level
//     A  z(rows rb) += X(rb, cb) y(cb),  y = b_own + children's update vectors (inverse maps);
//        the (0, 0) tile of a node also writes u = children's contributions to its halo
//     B  u(rows ab) -= L21(ab, cb) z(cb)
//   backward (root first), per level
//     C  w(cols cb) -= L21(ab, cb)^T x(halo rows ab)
//     D  x(cols jb) += X(ib, jb)^T (z / D + w)(ib)
// z, w and x start at zero (prologue).  Atomic accumulation makes the summation order, and so
// the last bits of the result, vary from run to run.
template <class T>
struct SolveArgs {
    int n;
    const int4* items;
    const int *f, *k, *own, *child0, *child1, *halo, *inv;
    const int64_t *front_off, *upd_off, *xinv_off, *halo_off, *inv_off;
    const T *pool, *xinv, *D, *b;
    T *x, *z, *w, *upd;
};

// sum of the children's update-vector entries that land on front position pos of node nd
template <class T>
__device__ __forceinline__ T mf_child_sum(const SolveArgs<T>& a, int nd, int pos, int q) {
    const int2 iv = reinterpret_cast<const int2*>(a.inv)[a.inv_off[nd] + pos];
    T s = T(0);
    if (iv.x >= 0) {
        const int c = a.child0[nd];
        s += __ldcg(a.upd + a.upd_off[c] + iv.x + (int64_t)(a.f[c] - a.k[c]) * q);
    }
    if (iv.y >= 0) {
        const int c = a.child1[nd];
        s += __ldcg(a.upd + a.upd_off[c] + iv.y + (int64_t)(a.f[c] - a.k[c]) * q);
    }
    return s;
}

template <class T>
__device__ __forceinline__ T mf_warp_sum(T v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Phase A tile (nd, rb, cb): rows i = rb*64 + warp + 8s, columns m = cb*64 + lane (+32).
template <class T, int NR>
__device__ __forceinline__ void mf_pt_own(const SolveArgs<T>& a, int4 it, T (*vs)[NB]) {
    const int nd = it.x, rb = it.y, cb = it.z;
    const int kN = a.k[nd], o = a.own[nd], n = a.n;
    const int r0 = rb * NB, c0 = cb * NB;
    for (int e = threadIdx.x; e < NR * NB; e += blockDim.x) {
        const int q = e / NB, m = e % NB, col = c0 + m;
        vs[q][m] = col < kN ? a.b[o + col + (int64_t)n * q] + mf_child_sum(a, nd, col, q) : T(0);
    }
    if (rb == 0 && cb == 0) {           // the node's halo starts as the children's contributions
        const int hN = a.f[nd] - kN;
        T* u = a.upd + a.upd_off[nd];
        for (int e = threadIdx.x; e < NR * hN; e += blockDim.x) {
            const int q = e / hN, r = e % hN;
            u[r + (int64_t)hN * q] = mf_child_sum(a, nd, kN + r, q);
        }
    }
    __syncthreads();
    const T* X = a.xinv + a.xinv_off[nd];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T xv[8][2];
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int i = r0 + warp + 8 * s;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int m = c0 + lane + 32 * h;
            xv[s][h] = (i < kN && m < kN && m <= i) ? X[(int64_t)i * kN + m] : T(0);
        }
    }
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int i = r0 + warp + 8 * s;
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            const T v = mf_warp_sum(xv[s][0] * vs[q][lane] + xv[s][1] * vs[q][lane + 32]);
            if (lane == 0 && i < kN) atomicAdd(a.z + o + i + (int64_t)n * q, v);
        }
    }
}

// Phase B tile (nd, ab, cb): halo rows r = ab*64 + lane (+32), columns j = cb*64 + warp + 8s.
template <class T, int NR>
__device__ __forceinline__ void mf_pt_halo(const SolveArgs<T>& a, int4 it, T (*vs)[NB], T (*part)[NR][NB]) {
    const int nd = it.x, ab = it.y, cb = it.z;
    const int fN = a.f[nd], kN = a.k[nd], hN = fN - kN, o = a.own[nd], n = a.n;
    const int r0 = ab * NB, c0 = cb * NB;
    for (int e = threadIdx.x; e < NR * NB; e += blockDim.x) {
        const int q = e / NB, m = e % NB, col = c0 + m;
        vs[q][m] = col < kN ? __ldcg(a.z + o + col + (int64_t)n * q) : T(0);
    }
    __syncthreads();
    const T* F = a.pool + a.front_off[nd] + kN;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T lv[8][2];
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int j = c0 + warp + 8 * s;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = r0 + lane + 32 * h;
            lv[s][h] = (j < kN && r < hN) ? F[(int64_t)j * fN + r] : T(0);
        }
    }
#pragma unroll
    for (int q = 0; q < NR; ++q)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            T acc = T(0);
#pragma unroll
            for (int s = 0; s < 8; ++s) acc += lv[s][h] * vs[q][warp + 8 * s];
            part[warp][q][lane + 32 * h] = acc;
        }
    __syncthreads();
    for (int e = threadIdx.x; e < NR * NB; e += blockDim.x) {
        const int q = e / NB, rl = e % NB, r = r0 + rl;
        if (r < hN) {
            T acc = T(0);
#pragma unroll
            for (int w = 0; w < 8; ++w) acc += part[w][q][rl];
            atomicAdd(a.upd + a.upd_off[nd] + r + (int64_t)hN * q, -acc);
        }
    }
}

// Phase C tile (nd, ab, cb): w(j) -= sum_r L21(r, j) x(halo r); lanes over rows, warps over columns.
template <class T, int NR>
__device__ __forceinline__ void mf_pt_bwd_z(const SolveArgs<T>& a, int4 it, T (*vs)[NB]) {
    const int nd = it.x, ab = it.y, cb = it.z;
    const int fN = a.f[nd], kN = a.k[nd], hN = fN - kN, o = a.own[nd], n = a.n;
    const int r0 = ab * NB, c0 = cb * NB;
    const int* hl = a.halo + a.halo_off[nd];
    for (int e = threadIdx.x; e < NR * NB; e += blockDim.x) {
        const int q = e / NB, rl = e % NB, r = r0 + rl;
        vs[q][rl] = r < hN ? __ldcg(a.x + hl[r] + (int64_t)n * q) : T(0);
    }
    __syncthreads();
    const T* F = a.pool + a.front_off[nd] + kN;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T lv[8][2];
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int j = c0 + warp + 8 * s;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = r0 + lane + 32 * h;
            lv[s][h] = (j < kN && r < hN) ? F[(int64_t)j * fN + r] : T(0);
        }
    }
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int j = c0 + warp + 8 * s;
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            const T v = mf_warp_sum(lv[s][0] * vs[q][lane] + lv[s][1] * vs[q][lane + 32]);
            if (lane == 0 && j < kN) atomicAdd(a.w + o + j + (int64_t)n * q, -v);
        }
    }
}

// Phase D tile (nd, ib, jb): x(j) += sum_i X(i, j) (z(i) / D(i) + w(i)); lanes over columns.
template <class T, int NR>
__device__ __forceinline__ void mf_pt_bwd_own(const SolveArgs<T>& a, int4 it, T (*vs)[NB], T (*part)[NR][NB]) {
    const int nd = it.x, ib = it.y, jb = it.z;
    const int kN = a.k[nd], o = a.own[nd], n = a.n;
    const int r0 = ib * NB, c0 = jb * NB;
    for (int e = threadIdx.x; e < NR * NB; e += blockDim.x) {
        const int q = e / NB, rl = e % NB, i = r0 + rl;
        vs[q][rl] = i < kN ? __ldcg(a.z + o + i + (int64_t)n * q) / a.D[o + i] + __ldcg(a.w + o + i + (int64_t)n * q) : T(0);
    }
    __syncthreads();
    const T* X = a.xinv + a.xinv_off[nd];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T xv[8][2];
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int i = r0 + warp + 8 * s;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = c0 + lane + 32 * h;
            xv[s][h] = (i < kN && j < kN && i >= j) ? X[(int64_t)i * kN + j] : T(0);
        }
    }
#pragma unroll
    for (int q = 0; q < NR; ++q)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            T acc = T(0);
#pragma unroll
            for (int s = 0; s < 8; ++s) acc += xv[s][h] * vs[q][warp + 8 * s];
            part[warp][q][lane + 32 * h] = acc;
        }
    __syncthreads();
    for (int e = threadIdx.x; e < NR * NB; e += blockDim.x) {
        const int q = e / NB, jl = e % NB, j = c0 + jl;
        if (j < kN) {
            T acc = T(0);
#pragma unroll
            for (int w = 0; w < 8; ++w) acc += part[w][q][jl];
            atomicAdd(a.x + o + j + (int64_t)n * q, acc);
        }
    }
}

template <class T, int NR>
__global__ void __launch_bounds__(SOLVE_THREADS) mf_solve_persistent_kernel(SolveArgs<T> a, SolveLevels lv) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ T vs[NR][NB];
    __shared__ T part[8][NR][NB];
    const int64_t nn = (int64_t)a.n * NR;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
        a.z[e] = T(0);
        a.w[e] = T(0);
        a.x[e] = T(0);
    }
    grid.sync();
    for (int L = 0; L < lv.nlev; ++L) {
        const int4* own = a.items + lv.own_off[L];
        for (int i = blockIdx.x; i < lv.own_cnt[L]; i += gridDim.x) {
            mf_pt_own<T, NR>(a, own[i], vs);
            __syncthreads();
        }
        grid.sync();
        if (lv.halo_cnt[L]) {
            const int4* hal = a.items + lv.halo_off[L];
            for (int i = blockIdx.x; i < lv.halo_cnt[L]; i += gridDim.x) {
                mf_pt_halo<T, NR>(a, hal[i], vs, part);
                __syncthreads();
            }
            grid.sync();
        }
    }
    for (int L = lv.nlev - 1; L >= 0; --L) {
        if (lv.halo_cnt[L]) {
            const int4* hal = a.items + lv.halo_off[L];
            for (int i = blockIdx.x; i < lv.halo_cnt[L]; i += gridDim.x) {
                mf_pt_bwd_z<T, NR>(a, hal[i], vs);
                __syncthreads();
            }
            grid.sync();
        }
        const int4* own = a.items + lv.own_off[L];
        for (int i = blockIdx.x; i < lv.own_cnt[L]; i += gridDim.x) {
            mf_pt_bwd_own<T, NR>(a, own[i], vs, part);
            __syncthreads();
        }
        if (L > 0) grid.sync();
    }
}

// ---- the same tile products as a dataflow schedule ---------------------------------------------
// One queue lists every tile of four phases in a topological order (forward: per level from the
// leaves, A then B; backward: per level from the root, C then D).  The forward sweep fans out:
// r starts as b, and a node's L21 z is subtracted straight from r at the node's halo rows (global
// dofs), so a node reads its right-hand side r(own) without gathering its children's update
// vectors:
//   A  z(rows rb) += X(rb, cb) r(own cols cb)            waits for the children's A and B
//   B  r(halo rows ab) -= L21(ab, cb) z(cb)              waits for the node's A
//   C  w(cols cb) -= L21(ab, cb)^T x(halo rows ab)       waits for the parent's D
//   D  x(cols jb) += X(ib, jb)^T (z / D + w)(ib)         waits for the node's A and C
// A node's A finds every contribution to its own rows in r once its children are complete: each
// child waited for its own children, so the whole subtree has subtracted.  The parent's D waited
// for its C, which waited for the grandparent's D, so C reads final x on every halo row.
// CTAs take tiles from the queue head in order; the earliest unfinished tile always has its
// inputs complete and a cooperative launch keeps every CTA resident, so the schedule cannot
// deadlock.  A tile loads its block of X or L21 (and its halo indices) before it waits: those do
// not depend on the solve, so their memory latency hides behind the wait.  Completion counters
// are raised with a fence + atomic add after the tile's __syncthreads and polled with ld.acquire;
// data written by other CTAs is read through L2 (__ldcg).  Every wait is bounded (clock64
// budget): on expiry the CTA writes NaN into the solution (NaN survives the later atomic
// additions), counts the tile as done and goes on, so the launch always ends and the caller sees
// a non-finite solution.
struct DataflowArgs {
    const int* queue;        // (phase << 29) | item index
    int qtotal;
    const int* own_tiles;    // per node: tiles of X (phases A, D)
    const int* halo_tiles;   // per node: tiles of L21 (phases B, C)
    const int* parent;
    int* cnt;                // 4 x nnodes completion counters, then the queue head
    int nnodes;
    int stall_node;          // test hook: this node's A never counts as complete (-1: off)
    long long wait_cycles;
};

__device__ __forceinline__ int mf_ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// spin until *p >= target; false when the budget ran out
__device__ __forceinline__ bool mf_wait_count(const int* p, int target, long long t0, long long budget) {
    for (unsigned it = 0;; ++it) {
        if (mf_ld_acquire(p) >= target) return true;
        if (clock64() - t0 > budget || it > (1u << 26)) return false;
        __nanosleep(64);
    }
}

// K partial sums per lane (K = 8, 16 or 32) reduced across the warp at once: at each exchange
// step a lane keeps one half of its values and receives the partner's sums of that half, so the
// K sums need K - 1 + log2(32 / K) shuffles instead of 5 K.  Afterwards lane l holds the warp
// total of value l >> log2(32 / K).
template <int K, class T>
__device__ __forceinline__ T mf_transpose_reduce(T (&v)[K], int lane) {
    static_assert(K == 8 || K == 16 || K == 32, "K must be 8, 16 or 32");
#pragma unroll
    for (int h = K / 2, o = 16; h >= 1; h >>= 1, o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const T send = up ? v[i] : v[i + h];
            const T keep = up ? v[i + h] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    T r = v[0];
#pragma unroll
    for (int o = 16 / K; o >= 1; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    return r;
}

__device__ __forceinline__ float mf_rcp(float d) { return __frcp_rn(d); }
__device__ __forceinline__ double mf_rcp(double d) { return __drcp_rn(d); }

__device__ __forceinline__ void mf_poison(float* p) { atomicExch(p, __int_as_float(0x7fffffff)); }
__device__ __forceinline__ void mf_poison(double* p) {
    atomicExch(reinterpret_cast<unsigned long long*>(p), 0x7fffffffffffffffULL);
}

template <class T, int NR>
__global__ void __launch_bounds__(SOLVE_THREADS) mf_solve_dataflow_kernel(SolveArgs<T> a, DataflowArgs d, T* r) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ T vs[NR][NB];
    __shared__ T part[8][NR][NB];
    __shared__ int s_q;
    const int64_t nn = (int64_t)a.n * NR;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
        r[e] = a.b[e];
        a.z[e] = T(0);
        a.w[e] = T(0);
        a.x[e] = T(0);
    }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e <= 4 * d.nnodes; e += gridDim.x * blockDim.x) d.cnt[e] = 0;
    grid.sync();
    int* cntA = d.cnt;
    int* cntB = d.cnt + d.nnodes;
    int* cntC = d.cnt + 2 * d.nnodes;
    int* cntD = d.cnt + 3 * d.nnodes;
    int* head = d.cnt + 4 * d.nnodes;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, n = a.n;
    for (;;) {
        if (threadIdx.x == 0) s_q = atomicAdd(head, 1);
        __syncthreads();
        const int q = s_q;
        if (q >= d.qtotal) break;
        const int code = d.queue[q], phase = code >> 29;
        const int4 it = a.items[code & ((1 << 29) - 1)];
        const int nd = it.x, kN = a.k[nd], fN = a.f[nd], hN = fN - kN, o = a.own[nd];
        const int r0 = it.y * NB, c0 = it.z * NB;
        // 1. the tile's block of X (A, D) or L21 (B, C) and its halo indices, before the wait
        T m[8][2];
        int hrow = 0;
        if (phase == 0 || phase == 3) {
            const T* X = a.xinv + a.xinv_off[nd];
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                const int i = r0 + warp + 8 * s;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int j = c0 + lane + 32 * h;
                    m[s][h] = (i < kN && j < kN && j <= i) ? X[(int64_t)i * kN + j] : T(0);
                }
            }
        } else {
            const T* F = a.pool + a.front_off[nd] + kN;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                const int j = c0 + warp + 8 * s;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int rr = r0 + lane + 32 * h;
                    m[s][h] = (j < kN && rr < hN) ? F[(int64_t)j * fN + rr] : T(0);
                }
            }
            const int rl = threadIdx.x % NB;
            if (threadIdx.x < NR * NB && r0 + rl < hN) hrow = a.halo[a.halo_off[nd] + r0 + rl];
        }
        // 2. wait for the tiles this one reads
        if (threadIdx.x == 0) {
            const long long t0 = clock64();
            bool ok = true;
            if (phase == 0) {
                const int c[2] = {a.child0[nd], a.child1[nd]};
                for (int h = 0; h < 2; ++h)
                    if (c[h] >= 0) {
                        const int needA = d.own_tiles[c[h]] + (c[h] == d.stall_node ? 1 : 0);
                        ok = ok && mf_wait_count(cntA + c[h], needA, t0, d.wait_cycles);
                        ok = ok && mf_wait_count(cntB + c[h], d.halo_tiles[c[h]], t0, d.wait_cycles);
                    }
            } else if (phase == 1) {
                ok = mf_wait_count(cntA + nd, d.own_tiles[nd], t0, d.wait_cycles);
            } else if (phase == 2) {
                const int p = d.parent[nd];   // a node with halo rows has a parent
                ok = p >= 0 && mf_wait_count(cntD + p, d.own_tiles[p], t0, d.wait_cycles);
            } else {
                ok = mf_wait_count(cntA + nd, d.own_tiles[nd], t0, d.wait_cycles) &&
                     mf_wait_count(cntC + nd, d.halo_tiles[nd], t0, d.wait_cycles);
            }
            if (!ok)
#pragma unroll
                for (int rr = 0; rr < NR; ++rr) mf_poison(a.x + (int64_t)n * rr);
        }
        __syncthreads();
        // 3. the vector part, then the tile product
        if (threadIdx.x < NR * NB) {
            const int qq = threadIdx.x / NB, e = threadIdx.x % NB;
            T v = T(0);
            if (phase == 0) {
                if (c0 + e < kN) v = __ldcg(r + o + c0 + e + (int64_t)n * qq);
            } else if (phase == 1) {
                if (c0 + e < kN) v = __ldcg(a.z + o + c0 + e + (int64_t)n * qq);
            } else if (phase == 2) {
                if (r0 + e < hN) v = __ldcg(a.x + hrow + (int64_t)n * qq);
            } else {
                const int i = r0 + e;
                if (i < kN) v = __ldcg(a.z + o + i + (int64_t)n * qq) * mf_rcp(a.D[o + i]) + __ldcg(a.w + o + i + (int64_t)n * qq);
            }
            vs[qq][e] = v;
        }
        __syncthreads();
        if (phase == 0 || phase == 2) {
            // lanes over the tile's columns: a warp sum per row (A) or column (C) of the warp's
            // eight and right-hand side, all reduced together
            constexpr int K = 8 * NR, SH = NR == 1 ? 2 : NR == 2 ? 1 : 0;
            T pv[K];
#pragma unroll
            for (int s = 0; s < 8; ++s)
#pragma unroll
                for (int qq = 0; qq < NR; ++qq) pv[s * NR + qq] = m[s][0] * vs[qq][lane] + m[s][1] * vs[qq][lane + 32];
            const T v = mf_transpose_reduce<K>(pv, lane);
            if ((lane & ((1 << SH) - 1)) == 0) {
                const int idx = lane >> SH, s = idx / NR, qq = idx % NR;
                if (phase == 0) {
                    const int i = r0 + warp + 8 * s;
                    if (i < kN) atomicAdd(a.z + o + i + (int64_t)n * qq, v);
                } else {
                    const int j = c0 + warp + 8 * s;
                    if (j < kN) atomicAdd(a.w + o + j + (int64_t)n * qq, -v);
                }
            }
        } else {
            // warps over the tile's rows (B: own columns j, D: rows i), partial sums in shared memory
#pragma unroll
            for (int qq = 0; qq < NR; ++qq)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    T acc = T(0);
#pragma unroll
                    for (int s = 0; s < 8; ++s) acc += m[s][h] * vs[qq][warp + 8 * s];
                    part[warp][qq][lane + 32 * h] = acc;
                }
            __syncthreads();
            if (threadIdx.x < NR * NB) {
                const int qq = threadIdx.x / NB, e = threadIdx.x % NB;
                T acc = T(0);
#pragma unroll
                for (int w = 0; w < 8; ++w) acc += part[w][qq][e];
                if (phase == 1) {
                    if (r0 + e < hN) atomicAdd(r + hrow + (int64_t)n * qq, -acc);
                } else {
                    if (c0 + e < kN) atomicAdd(a.x + o + c0 + e + (int64_t)n * qq, acc);
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // release: the CTA's atomics (ordered before this thread by the barrier) become visible
            // at GPU scope before the count does
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            atomicAdd((phase == 0 ? cntA : phase == 1 ? cntB : phase == 2 ? cntC : cntD) + nd, 1);
        }
    }
}

template <class T>
__global__ void mf_stability_kernel(int n, const T* __restrict__ D, double* out_min, unsigned long long* out_neg) {
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

constexpr size_t gemm_smem(size_t elem) { return 2 * elem * NB * NBP + elem * NB; }

}  // namespace

template <class T>
MultifrontalT<T>::MultifrontalT(const NDTree& Tr, const std::vector<int>& rowptr, const std::vector<int>& cols,
                                cudaStream_t stream)
    : stream_(stream) {
    n_ = Tr.nfree;
    nnodes_ = (int)Tr.nodes.size();
    flops_ = Tr.factor_flops();
    std::vector<int> f(nnodes_), k(nnodes_), own(nnodes_), parent(nnodes_), c0(nnodes_), c1(nnodes_);
    std::vector<int64_t> front_off(nnodes_), linv_off(nnodes_), ws_off(nnodes_), upd_off(nnodes_),
        halo_off(nnodes_), map_off(nnodes_), xinv_off(nnodes_);
    int64_t xo = 0;
    std::vector<int> halo_all, map_all;
    int64_t fo = 0, lo = 0, wo = 0, uo = 0;
    for (int i = 0; i < nnodes_; ++i) {
        const NDNode& nd = Tr.nodes[i];
        f[i] = nd.f(); k[i] = nd.k; own[i] = nd.own_start; parent[i] = nd.parent;
        c0[i] = nd.child[0]; c1[i] = nd.child[1];
        front_off[i] = fo; fo += (int64_t)f[i] * f[i];
        linv_off[i] = lo; lo += (int64_t)((nd.k + NB - 1) / NB) * NB * NB;
        xinv_off[i] = xo; xo += (int64_t)nd.k * nd.k;
        ws_off[i] = wo; wo += (int64_t)f[i] * NB;
        upd_off[i] = uo; uo += (int64_t)nd.h() * MF_MAX_RHS;
        halo_off[i] = (int64_t)halo_all.size();
        halo_all.insert(halo_all.end(), nd.halo.begin(), nd.halo.end());
        map_off[i] = (int64_t)map_all.size();
        map_all.insert(map_all.end(), Tr.parent_map[i].begin(), Tr.parent_map[i].end());
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
                        int nd = Tr.node_of[C];
                        int lc = C - Tr.nodes[nd].own_start;
                        int lr = Tr.local_index(nd, R);
                        if (lr < 0) { bad[t] = 1; return; }
                        fpos[e] = front_off[nd] + (int64_t)lc * f[nd] + lr;
                    }
            });
        for (auto& th : pool) th.join();
        for (int b : bad)
            if (b) throw std::logic_error("multifrontal: matrix entry outside its front");
    }
    // levels and work lists
    nlevels_ = Tr.max_height + 1;
    level_nodes_.assign(nlevels_, {});
    for (int i = 0; i < nnodes_; ++i) level_nodes_[Tr.nodes[i].height].push_back(i);
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
                for (int ti = 0; ti < ntr; ++ti) items.push_back(make_int4(nd, ti, 0, 0));
            }
            marks.push_back({L, 3, 0, t, b, items.size()});
            b = items.size();
            for (int nd : ln) {
                if (k[nd] <= t * NB) continue;
                int cc1 = t * NB + std::min(NB, k[nd] - t * NB);
                int ntr = (f[nd] - cc1 + NB - 1) / NB;
                for (int ti = 1; ti < ntr; ++ti)
                    for (int tj = 1; tj <= ti; ++tj) items.push_back(make_int4(nd, ti, tj, 0));
            }
            marks.push_back({L, 5, 0, t, b, items.size()});
        }
        size_t b = items.size();
        for (int nd : ln) items.push_back(make_int4(nd, 0, 0, 0));
        marks.push_back({L, 4, 0, 0, b, items.size()});
        b = items.size();
        for (int nd : ln)
            for (int rb = 0; rb * NB < k[nd]; ++rb) items.push_back(make_int4(nd, rb, 0, 0));
        marks.push_back({L, 6, 0, 0, b, items.size()});
        b = items.size();
        for (int nd : ln)
            for (int ab = 0; ab * NB < f[nd] - k[nd]; ++ab) items.push_back(make_int4(nd, ab, 0, 0));
        marks.push_back({L, 7, 0, 0, b, items.size()});
        // persistent-solve tiles: lower-triangular 64x64 blocks of X (rb >= cb), all blocks of L21
        b = items.size();
        for (int nd : ln)
            for (int rb = 0; rb * NB < k[nd]; ++rb)
                for (int cb = 0; cb <= rb; ++cb) items.push_back(make_int4(nd, rb, cb, 0));
        marks.push_back({L, 10, 0, 0, b, items.size()});
        b = items.size();
        for (int nd : ln)
            for (int ab = 0; ab * NB < f[nd] - k[nd]; ++ab)
                for (int cb = 0; cb * NB < k[nd]; ++cb) items.push_back(make_int4(nd, ab, cb, 0));
        marks.push_back({L, 11, 0, 0, b, items.size()});
        int maxb = 0;
        for (int nd : ln) maxb = std::max(maxb, (k[nd] + NB - 1) / NB);
        levels_[L].xdiag.resize(maxb);
        levels_[L].xoff.resize(maxb);
        for (int bi = 0; bi < maxb; ++bi) {
            b = items.size();
            for (int nd : ln)
                if (bi * NB < k[nd]) items.push_back(make_int4(nd, bi, 0, 0));
            marks.push_back({L, 8, 0, bi, b, items.size()});
            b = items.size();
            for (int nd : ln)
                if (bi * NB < k[nd])
                    for (int bj = 0; bj < bi; ++bj) items.push_back(make_int4(nd, bi, bj, 0));
            marks.push_back({L, 9, 0, bi, b, items.size()});
        }
        for (int nd : ln) {
            levels_[L].max_f = std::max(levels_[L].max_f, f[nd]);
            levels_[L].max_k = std::max(levels_[L].max_k, k[nd]);
            levels_[L].max_h = std::max(levels_[L].max_h, f[nd] - k[nd]);
        }
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
            case 3: lv.steps[m.step].upd_next = w; break;
            case 5: lv.steps[m.step].upd_rest = w; break;
            case 6: lv.own_blocks = w; break;
            case 7: lv.halo_blocks = w; break;
            case 8: lv.xdiag[m.step] = w; break;
            case 9: lv.xoff[m.step] = w; break;
            case 10:
            case 11: break;                      // persistent-solve tiles (solve_levels_)
            default: lv.nodes = w; break;
        }
    }
    for (int L = 0; L < nlevels_; ++L) {
        for (const Step& st : levels_[L].steps) {
            kernel_launches[0] += st.diag.count > 0;
            kernel_launches[1] += st.panel.count > 0;
            kernel_launches[2] += (st.upd_next.count > 0) + (st.upd_rest.count > 0);
        }
    }
    // persistent solve: inverse child maps (front position -> child halo index, per child slot)
    // and the per-level own / halo block lists
    {
        std::vector<int64_t> inv_off(nnodes_);
        int64_t io = 0;
        for (int i = 0; i < nnodes_; ++i) { inv_off[i] = io; io += f[i]; }
        std::vector<int> inv((size_t)2 * std::max<int64_t>(io, 1), -1);
        for (int i = 0; i < nnodes_; ++i) {
            const int cs[2] = {c0[i], c1[i]};
            for (int sl = 0; sl < 2; ++sl) {
                const int c = cs[sl];
                if (c < 0) continue;
                const std::vector<int>& mp = Tr.parent_map[c];
                for (int a = 0; a < (int)mp.size(); ++a) inv[2 * (inv_off[i] + mp[a]) + sl] = a;
            }
        }
        d_inv_off_.upload(inv_off, stream_);
        d_inv_.upload(inv, stream_);
        if (nlevels_ > MF_MAX_LEVELS) throw std::invalid_argument("multifrontal: elimination tree too deep");
        solve_levels_ = new SolveLevels();
        solve_levels_->nlev = nlevels_;
        for (const Pending& m : marks) {
            if (m.kind == 10) { solve_levels_->own_off[m.level] = (int)m.begin; solve_levels_->own_cnt[m.level] = (int)(m.end - m.begin); }
            if (m.kind == 11) { solve_levels_->halo_off[m.level] = (int)m.begin; solve_levels_->halo_cnt[m.level] = (int)(m.end - m.begin); }
        }
        // every node with a halo needs an own tile (0, 0) to start its update vector
        for (int i = 0; i < nnodes_; ++i)
            if (k[i] == 0 && f[i] > 0) persistent_ok_ = false;
        // dataflow schedule: the queue in topological order and the tiles per node and phase
        std::vector<int> queue, own_t(nnodes_, 0), halo_t(nnodes_, 0);
        const SolveLevels& sl = *solve_levels_;
        if (items.size() >= (size_t(1) << 29)) persistent_ok_ = false;
        for (int L = 0; L < nlevels_; ++L) {
            for (int q = sl.own_off[L]; q < sl.own_off[L] + sl.own_cnt[L]; ++q) {
                queue.push_back(q);
                ++own_t[items[q].x];
            }
            for (int q = sl.halo_off[L]; q < sl.halo_off[L] + sl.halo_cnt[L]; ++q) {
                queue.push_back((1 << 29) | q);
                ++halo_t[items[q].x];
            }
        }
        for (int L = nlevels_ - 1; L >= 0; --L) {
            for (int q = sl.halo_off[L]; q < sl.halo_off[L] + sl.halo_cnt[L]; ++q) queue.push_back((2 << 29) | q);
            for (int q = sl.own_off[L]; q < sl.own_off[L] + sl.own_cnt[L]; ++q) queue.push_back((3 << 29) | q);
        }
        df_qtotal_ = (int)queue.size();
        df_queue_.upload(queue, stream_);
        df_own_t_.upload(own_t, stream_);
        df_halo_t_.upload(halo_t, stream_);
        df_cnt_.alloc((size_t)4 * nnodes_ + 1);
        df_r_.alloc((size_t)std::max(n_, 1) * MF_MAX_RHS);
        if (const char* e = std::getenv("KLSA_SOLVE_STALL_NODE")) {
            // the k-th leaf of the elimination tree (a leaf has a parent unless the tree is one node)
            const auto& leaves = level_nodes_[0];
            const int kk = std::max(0, std::atoi(e));
            if (!leaves.empty()) df_stall_node_ = leaves[std::min<size_t>(kk, leaves.size() - 1)];
        }
    }
    d_f_.upload(f, stream_); d_k_.upload(k, stream_); d_own_.upload(own, stream_); d_parent_.upload(parent, stream_);
    d_child0_.upload(c0, stream_); d_child1_.upload(c1, stream_);
    d_front_off_.upload(front_off, stream_); d_linv_off_.upload(linv_off, stream_); d_ws_off_.upload(ws_off, stream_);
    d_upd_off_.upload(upd_off, stream_); d_halo_off_.upload(halo_off, stream_); d_map_off_.upload(map_off, stream_);
    d_xinv_off_.upload(xinv_off, stream_);
    xinv_.alloc(std::max<int64_t>(xo, 1));
    d_halo_.upload(halo_all, stream_); d_map_.upload(map_all, stream_);
    d_fpos_.upload(fpos, stream_);
    pool_.alloc(std::max<int64_t>(fo, 1));
    linv_.alloc(std::max<int64_t>(lo, 1));
    ws_half_ = wo;
    ws_.alloc(std::max<int64_t>(2 * wo, 1));
    KL_CUDA(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
    KL_CUDA(cudaEventCreateWithFlags(&ev_panel_, cudaEventDisableTiming));
    KL_CUDA(cudaEventCreateWithFlags(&ev_rest_, cudaEventDisableTiming));
    upd_.alloc(std::max<int64_t>(uo, 1));
    D_.alloc(std::max(n_, 1));
    y_.alloc((size_t)std::max(n_, 1) * MF_MAX_RHS);
    z_.alloc((size_t)std::max(n_, 1) * MF_MAX_RHS);
    KL_CUDA(cudaStreamCreateWithFlags(&inv_stream_, cudaStreamNonBlocking));
    KL_CUDA(cudaEventCreateWithFlags(&ev_level_, cudaEventDisableTiming));
    KL_CUDA(cudaEventCreateWithFlags(&ev_inv_, cudaEventDisableTiming));
    status_.alloc(1);
    status_.zero(stream_);
    int mk = 0, mh = 0;
    for (const Level& lv : levels_) { mk = std::max(mk, lv.max_k); mh = std::max(mh, lv.max_h); }
    const size_t smk = (size_t)mk * MF_MAX_RHS * sizeof(T), smh = (size_t)mh * MF_MAX_RHS * sizeof(T);
    if (std::max(smk, smh) > (size_t)200 * 1024)
        throw std::invalid_argument("multifrontal: separator too large for the shared-memory solve kernels");
    const int ak = (int)std::max<size_t>(smk, 48 * 1024), ah = (int)std::max<size_t>(smh, 48 * 1024);
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_own_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ak));
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_own_kernel<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, ak));
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_own_kernel<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, ak));
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_halo_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ak));
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_halo_kernel<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, ak));
    KL_CUDA(cudaFuncSetAttribute(mf_fwd_halo_kernel<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, ak));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_z_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ah));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_z_kernel<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, ah));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_z_kernel<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, ah));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_own_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ak));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_own_kernel<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, ak));
    KL_CUDA(cudaFuncSetAttribute(mf_bwd_own_kernel<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, ak));
    {
        // persistent solve: one CTA set resident on every SM (cooperative launch), shared memory
        // for the largest own or halo part
        int dev = 0, sms = 0;
        KL_CUDA(cudaGetDevice(&dev));
        KL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        int coop = 0;
        KL_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        int cap = 4;
        if (const char* e = std::getenv("KLSA_SOLVE_CTAS_PER_SM")) cap = std::max(1, std::atoi(e));
        const void* fns[3] = {(const void*)mf_solve_persistent_kernel<T, 1>, (const void*)mf_solve_persistent_kernel<T, 2>,
                              (const void*)mf_solve_persistent_kernel<T, 4>};
        const int nrs[3] = {1, 2, 4};
        const void* dfs[3] = {(const void*)mf_solve_dataflow_kernel<T, 1>, (const void*)mf_solve_dataflow_kernel<T, 2>,
                              (const void*)mf_solve_dataflow_kernel<T, 4>};
        for (int v = 0; v < 3; ++v) {
            (void)nrs;
            ps_smem_[v] = 0;
            int bps = 0;
            KL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fns[v], SOLVE_THREADS, ps_smem_[v]));
            ps_grid_[v] = coop ? sms * std::min(bps, cap) : 0;
            bps = 0;
            KL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, dfs[v], SOLVE_THREADS, 0));
            df_grid_[v] = coop ? sms * std::min(bps, cap) : 0;
        }
    }
    const int gsm = (int)gemm_smem(sizeof(T));
    KL_CUDA(cudaFuncSetAttribute(mf_panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, gsm));
    KL_CUDA(cudaFuncSetAttribute(mf_update_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, gsm));
    if constexpr (std::is_same<T, float>::value) {
        const char* e = std::getenv("KLSA_UPDATE_KERNEL");
        update_tc_ = e && std::string(e) == "tc";
        if (update_tc_)
            KL_CUDA(cudaFuncSetAttribute(mf_update_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
    }
    KL_CUDA(cudaFuncSetAttribute(mf_xoff_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, gsm));
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
template <class T>
template <class Fn>
void MultifrontalT<T>::replay(GraphSlot& slot, const void* key0, const void* key1, Fn&& launches) {
    if (g_timer.enabled || !graphs_enabled()) {
        launches();
        return;
    }
    if (!slot.exec || slot.key0 != key0 || slot.key1 != key1) {
        if (slot.exec) cudaGraphExecDestroy(slot.exec);
        slot.exec = nullptr;
        CaptureCount cc;
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
        slot.kernels = cc.n;
        slot.key0 = key0;
        slot.key1 = key1;
    }
    KL_CUDA(cudaGraphLaunch(slot.exec, stream_));
    count_launch(slot.kernels);
}

template <class T>
MultifrontalT<T>::~MultifrontalT() {
    delete solve_levels_;
    for (GraphSlot* s : {&fact_graph_, &solve_graph_[0], &solve_graph_[1], &solve_graph_[2]})
        if (s->exec) cudaGraphExecDestroy(s->exec);
    if (ev_panel_) cudaEventDestroy(ev_panel_);
    if (ev_rest_) cudaEventDestroy(ev_rest_);
    if (ev_level_) cudaEventDestroy(ev_level_);
    if (ev_inv_) cudaEventDestroy(ev_inv_);
    if (side_) cudaStreamDestroy(side_);
    if (inv_stream_) cudaStreamDestroy(inv_stream_);
}

template <class T>
void MultifrontalT<T>::factorize_async(const T* d_vals) {
    if (!d_vals && nnz_ > 0) throw std::logic_error("multifrontal: no matrix values");
    ++generation_;
    replay(fact_graph_, d_vals, nullptr, [&] { factorize_launches(d_vals); });
}

// trailing-update tiles of one step: CUDA-core tiles; with KLSA_UPDATE_KERNEL=tc and FP32 fronts
// the tensor-core tiles (tcgen05, 3xTF32)
template <class T>
void MultifrontalT<T>::launch_update(const MFWork& w, int t, const T* W, cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        if (update_tc_) {
            mf_update_tc_kernel<<<w.count, TC_THREADS, TC_SMEM, s>>>(w.items, t, d_f_.get(), d_k_.get(), d_front_off_.get(),
                                                                   d_ws_off_.get(), pool_.get(), W, status_.get());
            return;
        }
    }
    mf_update_kernel<T><<<w.count, 256, gemm_smem(sizeof(T)), s>>>(w.items, t, d_f_.get(), d_k_.get(), d_front_off_.get(),
                                                                  d_ws_off_.get(), pool_.get(), W);
}

template <class T>
void MultifrontalT<T>::factorize_launches(const T* d_vals) {
    KL_CUDA(cudaMemsetAsync(pool_.get(), 0, pool_.size() * sizeof(T), stream_));
    KL_CUDA(cudaMemsetAsync(status_.get(), 0, sizeof(int), stream_));
    if (nnz_ > 0) {
        mf_scatter_kernel<T><<<ceil_div(nnz_, 256), 256, 0, stream_>>>(nnz_, d_fpos_.get(), d_vals, pool_.get());
        count_launch();
    }
    // Look-ahead: step t's update of the tiles beyond the next pivot block runs on side_,
    // concurrently with step t+1's diagonal and panel; the next-block update waits for it.
    bool rest_inflight = false;
    auto join_rest = [&] {
        if (rest_inflight) KL_CUDA(cudaStreamWaitEvent(stream_, ev_rest_, 0));
        rest_inflight = false;
    };
    for (int L = 0; L < nlevels_; ++L) {
        Level& lv = levels_[L];
        join_rest();
        for (int s = 0; s < 2; ++s)
            if (lv.ea[s].count) {
                mf_extend_add_kernel<T><<<lv.ea[s].count, 256, 0, stream_>>>(lv.ea[s].items, d_f_.get(), d_k_.get(),
                                                                          d_parent_.get(), d_front_off_.get(),
                                                                          d_map_off_.get(), d_map_.get(), pool_.get());
                count_launch();
            }
        for (Step& st : lv.steps) {
            if (st.diag.count) {
                cudaEvent_t evk = g_timer.begin(stream_);
                mf_diag_kernel<T><<<st.diag.count, DIAG_THREADS, 0, stream_>>>(st.diag.items, st.t, d_f_.get(), d_k_.get(),
                                                                       d_own_.get(), d_front_off_.get(),
                                                                       d_linv_off_.get(), pool_.get(), D_.get(),
                                                                       linv_.get(), status_.get());
                g_timer.end(stream_, 5, evk);
                count_launch();
            }
            // block row st.t of the node inverses: needs this step's tile inverse and the panels
            // of the earlier steps only, so it runs on inv_stream_ beside the remaining steps
            if (st.t < (int)lv.xdiag.size() && lv.xdiag[st.t].count) {
                KL_CUDA(cudaEventRecord(ev_level_, stream_));
                KL_CUDA(cudaStreamWaitEvent(inv_stream_, ev_level_, 0));
                mf_xdiag_kernel<T><<<lv.xdiag[st.t].count, 256, 0, inv_stream_>>>(
                    lv.xdiag[st.t].items, d_k_.get(), d_linv_off_.get(), d_xinv_off_.get(), linv_.get(), xinv_.get());
                count_launch();
                if (lv.xoff[st.t].count) {
                    mf_xoff_kernel<T><<<lv.xoff[st.t].count, 256, gemm_smem(sizeof(T)), inv_stream_>>>(
                        lv.xoff[st.t].items, d_f_.get(), d_k_.get(), d_front_off_.get(), d_linv_off_.get(),
                        d_xinv_off_.get(), pool_.get(), linv_.get(), xinv_.get());
                    count_launch();
                }
            }
            T* W = ws_.get() + (st.t & 1) * ws_half_;
            if (st.panel.count) {
                cudaEvent_t evk = g_timer.begin(stream_);
                mf_panel_kernel<T><<<st.panel.count, 256, gemm_smem(sizeof(T)), stream_>>>(
                    st.panel.items, st.t, d_f_.get(), d_k_.get(), d_front_off_.get(), d_linv_off_.get(),
                    d_ws_off_.get(), pool_.get(), linv_.get(), W);
                g_timer.end(stream_, 6, evk);
                count_launch();
            }
            // the previous step's far update must finish before this step's updates start
            join_rest();
            if (st.upd_rest.count) {
                KL_CUDA(cudaEventRecord(ev_panel_, stream_));
                KL_CUDA(cudaStreamWaitEvent(side_, ev_panel_, 0));
                cudaEvent_t evk = g_timer.begin(side_);
                launch_update(st.upd_rest, st.t, W, side_);
                g_timer.end(side_, 4, evk);
                count_launch();
                KL_CUDA(cudaEventRecord(ev_rest_, side_));
                rest_inflight = true;
            }
            if (st.upd_next.count) {
                cudaEvent_t evk = g_timer.begin(stream_);
                launch_update(st.upd_next, st.t, W, stream_);
                g_timer.end(stream_, 4, evk);
                count_launch();
            }
        }
    }
    join_rest();
    KL_CUDA(cudaEventRecord(ev_inv_, inv_stream_));
    KL_CUDA(cudaStreamWaitEvent(stream_, ev_inv_, 0));
    KL_CHECK_LAUNCH();
}

template <class T>
int MultifrontalT<T>::read_status() {
    int st = 0;
    KL_CUDA(cudaMemcpyAsync(&st, status_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
    KL_CUDA(cudaStreamSynchronize(stream_));
    return st ? ST_SOLVER_ERROR : ST_SUCCESS;
}

template <class T>
int MultifrontalT<T>::factorize(const T* d_vals, bool check_status) {
    factorize_async(d_vals);
    return check_status ? read_status() : ST_SUCCESS;
}

template <class T>
template <int NR>
void MultifrontalT<T>::solve_impl(const T* d_b, T* d_x) {
    for (int L = 0; L < nlevels_; ++L) {
        Level& lv = levels_[L];
        const size_t smk = (size_t)lv.max_k * NR * sizeof(T);
        mf_fwd_gather_kernel<T, NR><<<lv.nodes.count, SOLVE_THREADS, 0, stream_>>>(
            lv.nodes.items, n_, d_f_.get(), d_k_.get(), d_own_.get(), d_child0_.get(), d_child1_.get(),
            d_upd_off_.get(), d_map_off_.get(), d_map_.get(), d_b, y_.get(), upd_.get());
        count_launch();
        if (lv.own_blocks.count) {
            mf_fwd_own_kernel<T, NR><<<lv.own_blocks.count, SOLVE_THREADS, smk, stream_>>>(
                lv.own_blocks.items, n_, d_k_.get(), d_own_.get(), d_xinv_off_.get(), xinv_.get(), y_.get(), z_.get());
            count_launch();
        }
        if (lv.halo_blocks.count) {
            mf_fwd_halo_kernel<T, NR><<<lv.halo_blocks.count, SOLVE_THREADS, smk, stream_>>>(
                lv.halo_blocks.items, n_, d_f_.get(), d_k_.get(), d_own_.get(), d_front_off_.get(), d_upd_off_.get(),
                pool_.get(), z_.get(), upd_.get());
            count_launch();
        }
    }
    for (int L = nlevels_ - 1; L >= 0; --L) {
        Level& lv = levels_[L];
        if (!lv.own_blocks.count) continue;
        const size_t smk = (size_t)lv.max_k * NR * sizeof(T), smh = (size_t)lv.max_h * NR * sizeof(T);
        mf_bwd_z_kernel<T, NR><<<lv.own_blocks.count, SOLVE_THREADS, smh, stream_>>>(
            lv.own_blocks.items, n_, d_f_.get(), d_k_.get(), d_own_.get(), d_front_off_.get(), d_halo_off_.get(),
            d_halo_.get(), pool_.get(), D_.get(), z_.get(), d_x, y_.get());
        count_launch();
        mf_bwd_own_kernel<T, NR><<<lv.own_blocks.count, SOLVE_THREADS, smk, stream_>>>(
            lv.own_blocks.items, n_, d_k_.get(), d_own_.get(), d_xinv_off_.get(), xinv_.get(), y_.get(), d_x);
        count_launch();
    }
    KL_CHECK_LAUNCH();
}

template <class T>
template <int NR>
void MultifrontalT<T>::solve_persistent(const T* d_b, T* d_x) {
    const int v = NR == 1 ? 0 : NR == 2 ? 1 : 2;
    SolveArgs<T> a;
    a.n = n_;
    a.items = items_.get();
    a.f = d_f_.get(); a.k = d_k_.get(); a.own = d_own_.get(); a.child0 = d_child0_.get(); a.child1 = d_child1_.get();
    a.halo = d_halo_.get(); a.inv = d_inv_.get();
    a.front_off = d_front_off_.get(); a.upd_off = d_upd_off_.get(); a.xinv_off = d_xinv_off_.get();
    a.halo_off = d_halo_off_.get(); a.inv_off = d_inv_off_.get();
    a.pool = pool_.get(); a.xinv = xinv_.get(); a.D = D_.get(); a.b = d_b;
    a.x = d_x; a.z = z_.get(); a.w = y_.get(); a.upd = upd_.get();
    const char* sel = std::getenv("KLSA_SOLVE_KERNEL");
    const bool barrier = sel && std::string(sel) == "barrier";
    if (!barrier && df_grid_[v] > 0) {
        DataflowArgs d;
        d.queue = df_queue_.get();
        d.qtotal = df_qtotal_;
        d.own_tiles = df_own_t_.get();
        d.halo_tiles = df_halo_t_.get();
        d.parent = d_parent_.get();
        d.cnt = df_cnt_.get();
        d.nnodes = nnodes_;
        d.stall_node = df_stall_node_;
        d.wait_cycles = 200000000LL;   // about 0.1 s at the GB300 SM clock
        T* rws = df_r_.get();
        void* args[3] = {&a, &d, &rws};
        KL_CUDA(cudaLaunchCooperativeKernel((const void*)mf_solve_dataflow_kernel<T, NR>, dim3(df_grid_[v]),
                                            dim3(SOLVE_THREADS), args, 0, stream_));
        count_launch();
        return;
    }
    void* args[2] = {&a, solve_levels_};
    KL_CUDA(cudaLaunchCooperativeKernel((const void*)mf_solve_persistent_kernel<T, NR>, dim3(ps_grid_[v]),
                                        dim3(SOLVE_THREADS), args, ps_smem_[v], stream_));
    count_launch();
}

template <class T>
bool MultifrontalT<T>::persistent_solve_enabled() const {
    const char* e = std::getenv("KLSA_SOLVE_KERNEL");
    const bool levels = e && std::string(e) == "levels";
    return !levels && persistent_ok_ && ps_grid_[0] > 0;
}

template <class T>
void MultifrontalT<T>::enqueue_factorize(const T* d_vals) {
    ++generation_;
    factorize_launches(d_vals);
}

template <class T>
void MultifrontalT<T>::enqueue_solve(const T* d_b, T* d_x) { solve_impl<1>(d_b, d_x); }

template <class T>
void MultifrontalT<T>::solve(const T* d_b, T* d_x, int nrhs) {
    // the persistent solve zeroes x before it reads b: an in-place call takes the level path
    if (persistent_solve_enabled() && d_b != d_x) {
        switch (nrhs) {
            case 1: solve_persistent<1>(d_b, d_x); return;
            case 2: solve_persistent<2>(d_b, d_x); return;
            case 3: solve_persistent<2>(d_b, d_x); solve_persistent<1>(d_b + 2 * (size_t)n_, d_x + 2 * (size_t)n_); return;
            case 4: solve_persistent<4>(d_b, d_x); return;
            default: throw std::invalid_argument("multifrontal solve: nrhs out of range");
        }
    }
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

template <class T>
void MultifrontalT<T>::stability(double* min_d, int64_t* negatives) {
    const int blocks = 64;
    DevBuf<double> mn(blocks);
    DevBuf<unsigned long long> ng(blocks);
    mf_stability_kernel<T><<<blocks, 256, 0, stream_>>>(n_, D_.get(), mn.get(), ng.get());
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

template class MultifrontalT<float>;
template class MultifrontalT<double>;

}  // namespace klsa
