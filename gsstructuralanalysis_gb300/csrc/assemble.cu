// assemble.cu -- Kirchhoff-Love shell tangent K(u), internal force Fint(u) and mass M on sm_103a.
//
// One warp per element.  Lane a (< (p+1)^2) owns control point a of the element: it loads the
// displacement once, forms its basis derivatives at each Gauss point, and the warp reduces the
// deformed base vectors / second derivatives with butterfly shuffles.  Every lane then
// evaluates the point's strains and stress resultants redundantly (scalar work), writes its
// control point's first-variation blocks to shared memory, and accumulates the 3x3 blocks of
// its assigned control-point pairs (A <= B) in registers across all Gauss points.
//
// Second variation of the bending strain (per dof pair r=(A,i), s=(B,j)), with ~a3 = a1 x a2,
// l = |~a3|, P_r = d~a3/du_r, q_r = a3.P_r, v = m^11 x,11 + m^22 x,22 + 2 m^12 x,12,
// c = v.a3, w = v - c a3, g_r = v.P_r, M_A = m^11 N_A,11 + m^22 N_A,22 + 2 m^12 N_A,12:
//   sum_ab w_ab d2b_ab = M_A (da3/du_s)_i + M_B (da3/du_r)_j
//                      + (N_A,1 N_B,2 - N_A,2 N_B,1) e_ijk w_k / l
//                      + (3c q_r q_s - g_r q_s - g_s q_r - c P_r.P_s) / l^2
// (the CPU oracle evaluates the same quantity from explicit vector derivatives instead).
#include <cuda_runtime.h>

#include <algorithm>
#include <utility>

#include "batch.h"
#include "df64.cuh"
#include "problem.h"

namespace klsa {

namespace {

template <class T> struct V3T { T x, y, z; };
template <class T> __device__ __forceinline__ V3T<T> mk(T a, T b, T c) { return {a, b, c}; }
template <class T> __device__ __forceinline__ T dot3(V3T<T> a, V3T<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> __device__ __forceinline__ V3T<T> cross3(V3T<T> a, V3T<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> __device__ __forceinline__ T comp(V3T<T> a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

template <class T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-control-point first-variation data in shared memory.
template <class T> struct CPData {
    T Bm[3][3];    // Bm[a][i]  = d eps_a / du_{A,i}
    T DBm[3][3];   // (t C Bm)[a][i]
    T Bb[3][3];    // Bb[a][i]  = d kappa_a / du_{A,i}
    T DBb[3][3];   // (t^3/12 C Bb)[a][i]
    T Da3[3][3];   // Da3[i][k] = (d a3 / du_{A,i})_k
    T Pv[3][3];    // Pv[i][k]  = (d ~a3 / du_{A,i})_k
    T q[3], g[3], h[3];
    T M, N1, N2;
};

template <int P> struct PairTable {
    static constexpr int NB = (P + 1) * (P + 1);
    static constexpr int NPAIR = NB * (NB + 1) / 2;
    static constexpr int NPS = (NPAIR + 31) / 32;
};

__constant__ unsigned char c_pairA[4][325];
__constant__ unsigned char c_pairB[4][325];

// Gauss-point state shared by all lanes (computed redundantly per lane).
template <class T> struct QPState {
    V3T<T> a1, a2, x11, x22, x12, a3, v, w;
    T il, il2, c;
    T n[3], m[3];
    T Cm[3][3], Cb[3][3];
    T dV;
};

// WITH_C: also keep the scaled material tensors t C and t^3/12 C (the tangent needs them; the
// residual needs only the stress resultants)
template <int P, class T, bool WITH_C = true>
__device__ __forceinline__ void qp_state(const double* __restrict__ geo, const T du[15], T tm, T tb, QPState<T>& s) {
    V3T<T> A1 = mk<T>(geo[0], geo[1], geo[2]), A2 = mk<T>(geo[3], geo[4], geo[5]);
    V3T<T> X11 = mk<T>(geo[6], geo[7], geo[8]), X22 = mk<T>(geo[9], geo[10], geo[11]), X12 = mk<T>(geo[12], geo[13], geo[14]);
    s.a1 = mk<T>(A1.x + du[0], A1.y + du[1], A1.z + du[2]);
    s.a2 = mk<T>(A2.x + du[3], A2.y + du[4], A2.z + du[5]);
    s.x11 = mk<T>(X11.x + du[6], X11.y + du[7], X11.z + du[8]);
    s.x22 = mk<T>(X22.x + du[9], X22.y + du[10], X22.z + du[11]);
    s.x12 = mk<T>(X12.x + du[12], X12.y + du[13], X12.z + du[14]);
    V3T<T> at = cross3(s.a1, s.a2);
    s.il = rsqrt(dot3(at, at));
    s.il2 = s.il * s.il;
    s.a3 = mk<T>(at.x * s.il, at.y * s.il, at.z * s.il);
    // membrane strain from displacement-gradient terms (avoids cancellation a.a - A.A)
    V3T<T> d1 = mk<T>(du[0], du[1], du[2]), d2 = mk<T>(du[3], du[4], du[5]);
    T e0 = dot3(A1, d1) + T(0.5) * dot3(d1, d1);
    T e1 = dot3(A2, d2) + T(0.5) * dot3(d2, d2);
    T e2 = dot3(A1, d2) + dot3(d1, A2) + dot3(d1, d2);
    // reference curvature coefficients X,ab.A3 precomputed per Gauss point
    T k0 = T(geo[22]) - dot3(s.x11, s.a3);
    T k1 = T(geo[23]) - dot3(s.x22, s.a3);
    T k2 = T(2) * (T(geo[24]) - dot3(s.x12, s.a3));
    T C00 = geo[15], C01 = geo[16], C02 = geo[17], C11 = geo[18], C12 = geo[19], C22 = geo[20];
    T C[3][3] = {{C00, C01, C02}, {C01, C11, C12}, {C02, C12, C22}};
    if constexpr (WITH_C) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) { s.Cm[a][b] = tm * C[a][b]; s.Cb[a][b] = tb * C[a][b]; }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            s.n[a] = s.Cm[a][0] * e0 + s.Cm[a][1] * e1 + s.Cm[a][2] * e2;
            s.m[a] = s.Cb[a][0] * k0 + s.Cb[a][1] * k1 + s.Cb[a][2] * k2;
        }
    } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            s.n[a] = tm * (C[a][0] * e0 + C[a][1] * e1 + C[a][2] * e2);
            s.m[a] = tb * (C[a][0] * k0 + C[a][1] * k1 + C[a][2] * k2);
        }
    }
    s.v = mk<T>(s.m[0] * s.x11.x + s.m[1] * s.x22.x + T(2) * s.m[2] * s.x12.x,
                s.m[0] * s.x11.y + s.m[1] * s.x22.y + T(2) * s.m[2] * s.x12.y,
                s.m[0] * s.x11.z + s.m[1] * s.x22.z + T(2) * s.m[2] * s.x12.z);
    s.c = dot3(s.v, s.a3);
    s.w = mk<T>(s.v.x - s.c * s.a3.x, s.v.y - s.c * s.a3.y, s.v.z - s.c * s.a3.z);
    s.dV = geo[21];
}

// First-variation data of one control point (basis derivatives N1,N2,N11,N22,N12).
template <class T>
__device__ __forceinline__ void cp_data(const QPState<T>& s, T N1, T N2, T N11, T N22, T N12, CPData<T>& o,
                                        bool stiffness) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        V3T<T> ei = mk<T>(i == 0, i == 1, i == 2);
        o.Bm[0][i] = N1 * comp(s.a1, i);
        o.Bm[1][i] = N2 * comp(s.a2, i);
        o.Bm[2][i] = N1 * comp(s.a2, i) + N2 * comp(s.a1, i);
        V3T<T> c1 = cross3(ei, s.a2), c2 = cross3(s.a1, ei);
        V3T<T> Pi = mk<T>(N1 * c1.x + N2 * c2.x, N1 * c1.y + N2 * c2.y, N1 * c1.z + N2 * c2.z);
        T qi = dot3(s.a3, Pi);
        V3T<T> Di = mk<T>((Pi.x - qi * s.a3.x) * s.il, (Pi.y - qi * s.a3.y) * s.il, (Pi.z - qi * s.a3.z) * s.il);
        T a3i = comp(s.a3, i);
        T db11 = N11 * a3i + dot3(s.x11, Di);
        T db22 = N22 * a3i + dot3(s.x22, Di);
        T db12 = N12 * a3i + dot3(s.x12, Di);
        o.Bb[0][i] = -db11;
        o.Bb[1][i] = -db22;
        o.Bb[2][i] = T(-2) * db12;
        if (stiffness) {
            o.Pv[i][0] = Pi.x; o.Pv[i][1] = Pi.y; o.Pv[i][2] = Pi.z;
            o.Da3[i][0] = Di.x; o.Da3[i][1] = Di.y; o.Da3[i][2] = Di.z;
            o.q[i] = qi;
            o.g[i] = dot3(s.v, Pi);
            o.h[i] = T(3) * s.c * qi - o.g[i];
        }
    }
    if (stiffness) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                o.DBm[a][i] = s.Cm[a][0] * o.Bm[0][i] + s.Cm[a][1] * o.Bm[1][i] + s.Cm[a][2] * o.Bm[2][i];
                o.DBb[a][i] = s.Cb[a][0] * o.Bb[0][i] + s.Cb[a][1] * o.Bb[1][i] + s.Cb[a][2] * o.Bb[2][i];
            }
        o.M = s.m[0] * N11 + s.m[1] * N22 + T(2) * s.m[2] * N12;
        o.N1 = N1;
        o.N2 = N2;
    }
}

// Tangent of element e by one warp (smw: the warp's shared-memory control-point records).
template <int P, class T>
__device__ __forceinline__ void tangent_element(int e, int m1, int n1, int ncp, int nq,
                                                const double* __restrict__ tab1, const double* __restrict__ tab2,
                                                const double* __restrict__ qpgeo, const double* __restrict__ ufull,
                                                double tmd, double tbd, T* __restrict__ elemK, CPData<T>* smw,
                                                int lane) {
    constexpr int NB1 = P + 1, NB = NB1 * NB1, D = 3 * NB;
    constexpr int NPS = PairTable<P>::NPS, NPAIR = PairTable<P>::NPAIR;
    const int e1 = e % m1, e2 = e / m1;
    const int la = lane % NB1, lb = lane / NB1;
    const bool own = lane < NB;
    T ux = 0, uy = 0, uz = 0;
    if (own) {
        int A = (e2 + lb) * n1 + (e1 + la);
        ux = (T)ufull[A]; uy = (T)ufull[ncp + A]; uz = (T)ufull[2 * ncp + A];
    }
    const T tm = (T)tmd, tb = (T)tbd;
    T acc[NPS][9];
#pragma unroll
    for (int s = 0; s < NPS; ++s)
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[s][k] = 0;
    for (int q2 = 0; q2 < nq; ++q2)
        for (int q1 = 0; q1 < nq; ++q1) {
            T N1 = 0, N2 = 0, N11 = 0, N22 = 0, N12 = 0;
            if (own) {
                const double* t1 = tab1 + (((size_t)e1 * nq + q1) * 3) * NB1;
                const double* t2 = tab2 + (((size_t)e2 * nq + q2) * 3) * NB1;
                T f0 = (T)t1[la], f1 = (T)t1[NB1 + la], f2 = (T)t1[2 * NB1 + la];
                T g0 = (T)t2[lb], g1 = (T)t2[NB1 + lb], g2 = (T)t2[2 * NB1 + lb];
                N1 = f1 * g0; N2 = f0 * g1; N11 = f2 * g0; N22 = f0 * g2; N12 = f1 * g1;
            }
            T du[15] = {N1 * ux, N1 * uy, N1 * uz, N2 * ux, N2 * uy, N2 * uz, N11 * ux, N11 * uy, N11 * uz,
                        N22 * ux, N22 * uy, N22 * uz, N12 * ux, N12 * uy, N12 * uz};
#pragma unroll
            for (int k = 0; k < 15; ++k) du[k] = warp_sum(du[k]);
            const double* geo = qpgeo + ((size_t)e * nq * nq + q2 * nq + q1) * QGEO;
            QPState<T> st;
            qp_state<P, T>(geo, du, tm, tb, st);
            if (own) cp_data<T>(st, N1, N2, N11, N22, N12, smw[lane], true);
            __syncwarp();
            const T dV = st.dV;
#pragma unroll
            for (int s = 0; s < NPS; ++s) {
                int pi = lane + 32 * s;
                if (pi >= NPAIR) break;
                const CPData<T>& A = smw[c_pairA[P - 1][pi]];
                const CPData<T>& B = smw[c_pairB[P - 1][pi]];
                T Sm = st.n[0] * A.N1 * B.N1 + st.n[1] * A.N2 * B.N2 + st.n[2] * (A.N1 * B.N2 + A.N2 * B.N1);
                T cr = (A.N1 * B.N2 - A.N2 * B.N1) * st.il;
                T wv[3] = {st.w.x, st.w.y, st.w.z};
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        T k = A.DBm[0][i] * B.Bm[0][j] + A.DBm[1][i] * B.Bm[1][j] + A.DBm[2][i] * B.Bm[2][j] +
                              A.DBb[0][i] * B.Bb[0][j] + A.DBb[1][i] * B.Bb[1][j] + A.DBb[2][i] * B.Bb[2][j];
                        if (i == j) k += Sm;
                        T pp = A.Pv[i][0] * B.Pv[j][0] + A.Pv[i][1] * B.Pv[j][1] + A.Pv[i][2] * B.Pv[j][2];
                        T gb = A.M * B.Da3[j][i] + B.M * A.Da3[i][j] +
                               st.il2 * (A.q[i] * B.h[j] - A.g[i] * B.q[j] - st.c * pp);
                        // e_ijk w_k
                        if (i != j) {
                            int kk = 3 - i - j;
                            T sgn = ((j - i + 3) % 3 == 1) ? T(1) : T(-1);
                            gb += cr * sgn * wv[kk];
                        }
                        acc[s][3 * i + j] += (k - gb) * dV;
                    }
            }
            __syncwarp();
        }
    T* Ke = elemK + (size_t)e * D * D;
#pragma unroll
    for (int s = 0; s < NPS; ++s) {
        int pi = lane + 32 * s;
        if (pi >= NPAIR) break;
        int a = c_pairA[P - 1][pi], b = c_pairB[P - 1][pi];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                Ke[(size_t)(3 * a + i) * D + 3 * b + j] = acc[s][3 * i + j];
                if (a != b) Ke[(size_t)(3 * b + j) * D + 3 * a + i] = acc[s][3 * i + j];
            }
    }
}


template <int P, class T>
__global__ void __launch_bounds__(128) kl_tangent_kernel(int nel, int m1, int n1, int ncp, int nq,
                                                         const double* __restrict__ tab1, const double* __restrict__ tab2,
                                                         const double* __restrict__ qpgeo,
                                                         const double* __restrict__ ufull, double tmd, double tbd,
                                                         T* __restrict__ elemK) {
    __shared__ CPData<T> sm[4][(P + 1) * (P + 1)];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int e = blockIdx.x * 4 + warp;
    if (e >= nel) return;
    tangent_element<P, T>(e, m1, n1, ncp, nq, tab1, tab2, qpgeo, ufull, tmd, tbd, elemK, sm[warp], lane);
}

// Instance of a flat work index: the largest k with off[k] <= g (off ascending, off[0] = 0).
__device__ __forceinline__ int find_segment(const int* __restrict__ off, int n, int g) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Persistent batched tangent (FP32): every warp walks the flat element list of all instances of
// degree P (instance list `insts`, element prefix sums `elem_off`) with a grid-stride loop.
template <int P>
__global__ void __launch_bounds__(128) kl_tangent_batch_kernel(int ninst, const int* __restrict__ insts,
                                                               const int* __restrict__ elem_off,
                                                               const BatchInst* __restrict__ desc) {
    __shared__ CPData<float> sm[4][(P + 1) * (P + 1)];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = elem_off[ninst];
    for (int g = blockIdx.x * 4 + warp; g < total; g += gridDim.x * 4) {
        const int k = find_segment(elem_off, ninst, g);
        const BatchInst& d = desc[insts[k]];
        tangent_element<P, float>(g - elem_off[k], d.m1, d.n1, d.ncp, d.nq, d.tab1, d.tab2, d.qpgeo, d.ufull, d.tm,
                                  d.tb, d.elemK, sm[warp], lane);
        __syncwarp();
    }
}

// Internal force in FP64.  A warp holds ES = 32 / max((p+1)^2, nq^2) elements: lanes first act
// as Gauss points (one lane evaluates one point's deformed geometry and stress resultants, no
// redundant per-lane work), then as control points (one lane accumulates one control point's
// three force components over the element's Gauss points, reading the point states from
// shared memory).
constexpr int QSTATE = 16;   // G1, G2, S11, S22, S12 of one Gauss point

// Internal forces of the elements of warp work unit `grp` (elements grp*es .. grp*es+es-1);
// usw / qsw: the warp's shared-memory displacement and Gauss-point records.
template <int P>
__device__ __forceinline__ void fint_group(int grp, int nel, int m1, int n1, int ncp, int nq,
                                           const double* __restrict__ tab1, const double* __restrict__ tab2,
                                           const double* __restrict__ qpgeo, const double* __restrict__ ufull,
                                           double tm, double tb, double* __restrict__ elemR, double (*usw)[3],
                                           double (*qsw)[QSTATE], int lane) {
    constexpr int NB1 = P + 1, NB = NB1 * NB1, D = 3 * NB;
    const int nqp = nq * nq;
    const int lpe = NB > nqp ? NB : nqp;
    const int es = 32 / lpe;
    const int slot = lane / lpe, idx = lane % lpe;
    const int e = grp * es + slot;
    const bool live = slot < es && e < nel;
    const int e1 = live ? e % m1 : 0, e2 = live ? e / m1 : 0;
    // phase 0: displacements of the element's control points
    if (live && idx < NB) {
        int A = (e2 + idx / NB1) * n1 + (e1 + idx % NB1);
        usw[slot * NB + idx][0] = ufull[A];
        usw[slot * NB + idx][1] = ufull[ncp + A];
        usw[slot * NB + idx][2] = ufull[2 * ncp + A];
    }
    __syncwarp();
    // phase 1: one lane per Gauss point
    if (live && idx < nqp) {
        int q1 = idx % nq, q2 = idx / nq;
        const double* t1 = tab1 + (((size_t)e1 * nq + q1) * 3) * NB1;
        const double* t2 = tab2 + (((size_t)e2 * nq + q2) * 3) * NB1;
        double du[15];
#pragma unroll
        for (int k = 0; k < 15; ++k) du[k] = 0.0;
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            int a = c % NB1, b = c / NB1;
            double N1 = t1[NB1 + a] * t2[b], N2 = t1[a] * t2[NB1 + b];
            double N11 = t1[2 * NB1 + a] * t2[b], N22 = t1[a] * t2[2 * NB1 + b], N12 = t1[NB1 + a] * t2[NB1 + b];
            const double* u = usw[slot * NB + c];
            double Ns[5] = {N1, N2, N11, N22, N12};
#pragma unroll
            for (int g = 0; g < 5; ++g) {
                du[3 * g] += Ns[g] * u[0];
                du[3 * g + 1] += Ns[g] * u[1];
                du[3 * g + 2] += Ns[g] * u[2];
            }
        }
        const double* geo = qpgeo + ((size_t)e * nqp + idx) * QGEO;
        QPState<double> st;
        qp_state<P, double, false>(geo, du, tm, tb, st);
        // f_{A,i} = sum_qp [N1 G1 + N2 G2 - N11 S11 - N22 S22 - N12 S12]_i with
        //   G1 = dV (n0 a1 + n2 a2 - (a2 x w)/l),  G2 = dV (n1 a2 + n2 a1 - (w x a1)/l),
        //   S11 = dV m0 a3, S22 = dV m1 a3, S12 = 2 dV m2 a3   (w = v - (v.a3) a3)
        const double dV = st.dV;
        V3T<double> u1 = cross3(st.a2, st.w), u2 = cross3(st.w, st.a1);
        double* o = qsw[slot * nqp + idx];
        o[0] = dV * (st.n[0] * st.a1.x + st.n[2] * st.a2.x - u1.x * st.il);
        o[1] = dV * (st.n[0] * st.a1.y + st.n[2] * st.a2.y - u1.y * st.il);
        o[2] = dV * (st.n[0] * st.a1.z + st.n[2] * st.a2.z - u1.z * st.il);
        o[3] = dV * (st.n[1] * st.a2.x + st.n[2] * st.a1.x - u2.x * st.il);
        o[4] = dV * (st.n[1] * st.a2.y + st.n[2] * st.a1.y - u2.y * st.il);
        o[5] = dV * (st.n[1] * st.a2.z + st.n[2] * st.a1.z - u2.z * st.il);
        const double s11 = dV * st.m[0], s22 = dV * st.m[1], s12 = 2.0 * dV * st.m[2];
        o[6] = s11 * st.a3.x; o[7] = s11 * st.a3.y; o[8] = s11 * st.a3.z;
        o[9] = s22 * st.a3.x; o[10] = s22 * st.a3.y; o[11] = s22 * st.a3.z;
        o[12] = s12 * st.a3.x; o[13] = s12 * st.a3.y; o[14] = s12 * st.a3.z;
    }
    __syncwarp();
    // phase 2: one lane per control point, 15 FMAs per Gauss point
    if (live && idx < NB) {
        int a = idx % NB1, b = idx / NB1;
        double f[3] = {0.0, 0.0, 0.0};
        for (int qq = 0; qq < nqp; ++qq) {
            int q1 = qq % nq, q2 = qq / nq;
            const double* t1 = tab1 + (((size_t)e1 * nq + q1) * 3) * NB1;
            const double* t2 = tab2 + (((size_t)e2 * nq + q2) * 3) * NB1;
            double N1 = t1[NB1 + a] * t2[b], N2 = t1[a] * t2[NB1 + b];
            double N11 = t1[2 * NB1 + a] * t2[b], N22 = t1[a] * t2[2 * NB1 + b], N12 = t1[NB1 + a] * t2[NB1 + b];
            const double* o = qsw[slot * nqp + qq];
#pragma unroll
            for (int i = 0; i < 3; ++i)
                f[i] += N1 * o[i] + N2 * o[3 + i] - N11 * o[6 + i] - N22 * o[9 + i] - N12 * o[12 + i];
        }
        for (int i = 0; i < 3; ++i) elemR[(size_t)e * D + 3 * idx + i] = f[i];
    }
}

// The same element group with the two long accumulations -- the displacement derivatives at a
// Gauss point (sum over control points of N u) and the control-point forces (sum over Gauss
// points of N times the point's stress terms) -- in double-float arithmetic (df64.cuh) on the
// FP32 pipes, from basis tables pre-split into FP32 hi/lo pairs (tab1s, tab2s).  The Gauss-point
// state (deformed geometry, strains, stress resultants) stays FP64.  The sums carry about 48
// significant bits: the residual's relative error stays near 1e-14, six orders of magnitude
// under the 1e-8 force tolerance it decides.
template <int P>
__device__ __forceinline__ void fint_group_df(int grp, int nel, int m1, int n1, int ncp, int nq,
                                              const float2* __restrict__ tab1s, const float2* __restrict__ tab2s,
                                              const double* __restrict__ qpgeo, const double* __restrict__ ufull,
                                              double tm, double tb, double* __restrict__ elemR, df2 (*usw)[3],
                                              df2 (*qsw)[15], int lane) {
    constexpr int NB1 = P + 1, NB = NB1 * NB1, D = 3 * NB;
    const int nqp = nq * nq;
    const int lpe = NB > nqp ? NB : nqp;
    const int es = 32 / lpe;
    const int slot = lane / lpe, idx = lane % lpe;
    const int e = grp * es + slot;
    const bool live = slot < es && e < nel;
    const int e1 = live ? e % m1 : 0, e2 = live ? e / m1 : 0;
    if (live && idx < NB) {
        const int A = (e2 + idx / NB1) * n1 + (e1 + idx % NB1);
        usw[slot * NB + idx][0] = df_split(ufull[A]);
        usw[slot * NB + idx][1] = df_split(ufull[ncp + A]);
        usw[slot * NB + idx][2] = df_split(ufull[2 * ncp + A]);
    }
    __syncwarp();
    if (live && idx < nqp) {
        const int q1 = idx % nq, q2 = idx / nq;
        df2 t1[3 * NB1], t2[3 * NB1];
        const float2* r1 = tab1s + (((size_t)e1 * nq + q1) * 3) * NB1;
        const float2* r2 = tab2s + (((size_t)e2 * nq + q2) * 3) * NB1;
#pragma unroll
        for (int k = 0; k < 3 * NB1; ++k) {
            const float2 a = r1[k], b = r2[k];
            t1[k] = {a.x, a.y};
            t2[k] = {b.x, b.y};
        }
        df2 du[15];
#pragma unroll
        for (int k = 0; k < 15; ++k) du[k] = {0.f, 0.f};
#pragma unroll
        for (int c = 0; c < NB; ++c) {
            const int a = c % NB1, b = c / NB1;
            const df2 Ns[5] = {df_mul(t1[NB1 + a], t2[b]), df_mul(t1[a], t2[NB1 + b]), df_mul(t1[2 * NB1 + a], t2[b]),
                               df_mul(t1[a], t2[2 * NB1 + b]), df_mul(t1[NB1 + a], t2[NB1 + b])};
            const df2* u = usw[slot * NB + c];
#pragma unroll
            for (int g = 0; g < 5; ++g) {
                df_fma(du[3 * g], Ns[g], u[0]);
                df_fma(du[3 * g + 1], Ns[g], u[1]);
                df_fma(du[3 * g + 2], Ns[g], u[2]);
            }
        }
        double dud[15];
#pragma unroll
        for (int k = 0; k < 15; ++k) dud[k] = df_to_double(du[k]);
        const double* geo = qpgeo + ((size_t)e * nqp + idx) * QGEO;
        QPState<double> st;
        qp_state<P, double, false>(geo, dud, tm, tb, st);
        const double dV = st.dV;
        V3T<double> u1 = cross3(st.a2, st.w), u2 = cross3(st.w, st.a1);
        df2* o = qsw[slot * nqp + idx];
        o[0] = df_split(dV * (st.n[0] * st.a1.x + st.n[2] * st.a2.x - u1.x * st.il));
        o[1] = df_split(dV * (st.n[0] * st.a1.y + st.n[2] * st.a2.y - u1.y * st.il));
        o[2] = df_split(dV * (st.n[0] * st.a1.z + st.n[2] * st.a2.z - u1.z * st.il));
        o[3] = df_split(dV * (st.n[1] * st.a2.x + st.n[2] * st.a1.x - u2.x * st.il));
        o[4] = df_split(dV * (st.n[1] * st.a2.y + st.n[2] * st.a1.y - u2.y * st.il));
        o[5] = df_split(dV * (st.n[1] * st.a2.z + st.n[2] * st.a1.z - u2.z * st.il));
        const double s11 = dV * st.m[0], s22 = dV * st.m[1], s12 = 2.0 * dV * st.m[2];
        o[6] = df_split(s11 * st.a3.x); o[7] = df_split(s11 * st.a3.y); o[8] = df_split(s11 * st.a3.z);
        o[9] = df_split(s22 * st.a3.x); o[10] = df_split(s22 * st.a3.y); o[11] = df_split(s22 * st.a3.z);
        o[12] = df_split(s12 * st.a3.x); o[13] = df_split(s12 * st.a3.y); o[14] = df_split(s12 * st.a3.z);
    }
    __syncwarp();
    if (live && idx < NB) {
        const int a = idx % NB1, b = idx / NB1;
        df2 f[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
        for (int qq = 0; qq < nqp; ++qq) {
            const int q1 = qq % nq, q2 = qq / nq;
            const float2* r1 = tab1s + (((size_t)e1 * nq + q1) * 3) * NB1;
            const float2* r2 = tab2s + (((size_t)e2 * nq + q2) * 3) * NB1;
            const float2 v0 = r1[a], v1 = r1[NB1 + a], v2 = r1[2 * NB1 + a];
            const float2 w0 = r2[b], w1 = r2[NB1 + b], w2 = r2[2 * NB1 + b];
            const df2 t10 = {v0.x, v0.y}, t11 = {v1.x, v1.y}, t12 = {v2.x, v2.y};
            const df2 t20 = {w0.x, w0.y}, t21 = {w1.x, w1.y}, t22 = {w2.x, w2.y};
            const df2 N1 = df_mul(t11, t20), N2 = df_mul(t10, t21), N11 = df_mul(t12, t20), N22 = df_mul(t10, t22),
                      N12 = df_mul(t11, t21);
            const df2* o = qsw[slot * nqp + qq];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                df_fma(f[i], N1, o[i]);
                df_fma(f[i], N2, o[3 + i]);
                df_fms(f[i], N11, o[6 + i]);
                df_fms(f[i], N22, o[9 + i]);
                df_fms(f[i], N12, o[12 + i]);
            }
        }
        for (int i = 0; i < 3; ++i) elemR[(size_t)e * D + 3 * idx + i] = df_to_double(f[i]);
    }
}

// FP32 pairs underflow below ~1e-38 (and lose their low word below ~1e-31): a warp whose
// elements' displacements are all nonzero and tiny (largest |u| under 1e-20, e.g. an iteration
// converging to the undeformed state) evaluates its elements in plain FP64 instead.
template <int P>
__device__ __forceinline__ bool fint_group_tiny(int grp, int nel, int m1, int n1, int ncp, int nq,
                                                const double* __restrict__ ufull, int lane) {
    constexpr int NB1 = P + 1, NB = NB1 * NB1;
    const int lpe = NB > nq * nq ? NB : nq * nq;
    const int slot = lane / lpe, idx = lane % lpe;
    const int e = grp * (32 / lpe) + slot;
    // the largest |u| of the warp's elements, compared through the high words of the doubles
    // (for non-negative doubles the bit patterns order as the values): integer pipes only
    auto hiw = [](double v) { return static_cast<unsigned>(__double_as_longlong(v) >> 32) & 0x7fffffffu; };
    unsigned m = 0;
    if (slot < 32 / lpe && e < nel && idx < NB) {
        const int e1 = e % m1, e2 = e / m1;
        const int A = (e2 + idx / NB1) * n1 + (e1 + idx % NB1);
        m = max(hiw(ufull[A]), max(hiw(ufull[ncp + A]), hiw(ufull[2 * ncp + A])));
    }
    m = __reduce_max_sync(0xffffffffu, m);
    return m != 0u && m < 0x3BC79CA1u;   // 0 < max |u| < 1e-20 (high word of 1e-20)
}

// shared memory of one warp, for either variant of the element group
union FintShared {
    struct { double us[32][3]; double qs[32][QSTATE]; } d;
    struct { df2 us[32][3]; df2 qs[32][15]; } f;
};

template <int P>
__device__ __forceinline__ void fint_group_auto(int grp, int nel, int m1, int n1, int ncp, int nq,
                                                const double* __restrict__ tab1, const double* __restrict__ tab2,
                                                const float2* __restrict__ tab1s, const float2* __restrict__ tab2s,
                                                const double* __restrict__ qpgeo, const double* __restrict__ ufull,
                                                double tm, double tb, double* __restrict__ elemR, FintShared& sh,
                                                int lane) {
    if (fint_group_tiny<P>(grp, nel, m1, n1, ncp, nq, ufull, lane))
        fint_group<P>(grp, nel, m1, n1, ncp, nq, tab1, tab2, qpgeo, ufull, tm, tb, elemR, sh.d.us, sh.d.qs, lane);
    else
        fint_group_df<P>(grp, nel, m1, n1, ncp, nq, tab1s, tab2s, qpgeo, ufull, tm, tb, elemR, sh.f.us, sh.f.qs, lane);
}

template <int P>
__global__ void __launch_bounds__(128, 6) kl_fint_df_kernel(int nel, int m1, int n1, int ncp, int nq,
                                                         const double* __restrict__ tab1,
                                                         const double* __restrict__ tab2,
                                                         const float2* __restrict__ tab1s,
                                                         const float2* __restrict__ tab2s,
                                                         const double* __restrict__ qpgeo,
                                                         const double* __restrict__ ufull, double tm, double tb,
                                                         double* __restrict__ elemR) {
    __shared__ FintShared sh[4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    fint_group_auto<P>(blockIdx.x * 4 + warp, nel, m1, n1, ncp, nq, tab1, tab2, tab1s, tab2s, qpgeo, ufull, tm, tb,
                       elemR, sh[warp], lane);
}

template <int P>
__global__ void __launch_bounds__(128) kl_fint_kernel(int nel, int m1, int n1, int ncp, int nq,
                                                      const double* __restrict__ tab1, const double* __restrict__ tab2,
                                                      const double* __restrict__ qpgeo, const double* __restrict__ ufull,
                                                      double tm, double tb, double* __restrict__ elemR) {
    __shared__ double us[4][32][3];
    __shared__ double qs[4][32][QSTATE];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    fint_group<P>(blockIdx.x * 4 + warp, nel, m1, n1, ncp, nq, tab1, tab2, qpgeo, ufull, tm, tb, elemR, us[warp],
                  qs[warp], lane);
}

// Persistent batched internal force: warps walk the flat list of element groups of all
// instances of degree P (group prefix sums `grp_off`).
template <int P>
__global__ void __launch_bounds__(128) kl_fint_batch_kernel(int ninst, const int* __restrict__ insts,
                                                            const int* __restrict__ grp_off,
                                                            const BatchInst* __restrict__ desc) {
    __shared__ FintShared sh[4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = grp_off[ninst];
    for (int g = blockIdx.x * 4 + warp; g < total; g += gridDim.x * 4) {
        const int k = find_segment(grp_off, ninst, g);
        const BatchInst& d = desc[insts[k]];
        fint_group_auto<P>(g - grp_off[k], d.nel, d.m1, d.n1, d.ncp, d.nq, d.tab1, d.tab2, d.tab1s, d.tab2s, d.qpgeo,
                           d.ufull, d.tm, d.tb, d.elemR, sh[warp], lane);
        __syncwarp();
    }
}

template <int P>
__global__ void __launch_bounds__(128) kl_mass_kernel(int nel, int m1, int nq, const double* __restrict__ tab1,
                                                      const double* __restrict__ tab2, const double* __restrict__ qpgeo,
                                                      double rhot, double* __restrict__ elemK) {
    constexpr int NB1 = P + 1, NB = NB1 * NB1, D = 3 * NB;
    constexpr int NPS = PairTable<P>::NPS, NPAIR = PairTable<P>::NPAIR;
    __shared__ double Ns[4][NB];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int e = blockIdx.x * 4 + warp;
    if (e >= nel) return;
    const int e1 = e % m1, e2 = e / m1;
    double acc[NPS];
    for (int s = 0; s < NPS; ++s) acc[s] = 0;
    for (int q2 = 0; q2 < nq; ++q2)
        for (int q1 = 0; q1 < nq; ++q1) {
            if (lane < NB) {
                const double* t1 = tab1 + (((size_t)e1 * nq + q1) * 3) * NB1;
                const double* t2 = tab2 + (((size_t)e2 * nq + q2) * 3) * NB1;
                Ns[warp][lane] = t1[lane % NB1] * t2[lane / NB1];
            }
            __syncwarp();
            double dV = qpgeo[((size_t)e * nq * nq + q2 * nq + q1) * QGEO + 21];
            for (int s = 0; s < NPS; ++s) {
                int pi = lane + 32 * s;
                if (pi < NPAIR) acc[s] += rhot * Ns[warp][c_pairA[P - 1][pi]] * Ns[warp][c_pairB[P - 1][pi]] * dV;
            }
            __syncwarp();
        }
    double* Ke = elemK + (size_t)e * D * D;
    for (int s = 0; s < NPS; ++s) {
        int pi = lane + 32 * s;
        if (pi >= NPAIR) break;
        int a = c_pairA[P - 1][pi], b = c_pairB[P - 1][pi];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double v = (i == j) ? acc[s] : 0.0;
                Ke[(size_t)(3 * a + i) * D + 3 * b + j] = v;
                Ke[(size_t)(3 * b + j) * D + 3 * a + i] = v;
            }
    }
}

// CSR gather: every nonzero (row R, col C) sums the element entries of the elements that
// contain both control points (tensor-product structure: element e covers points e..e+p).
// One warp per row; lanes over the row's columns.
template <class TE, class TV>
__global__ void csr_gather_kernel(int nfree, int64_t nnz, int p, int n1, int m1, int m2, int ncp,
                                  const int* __restrict__ rowptr, const int* __restrict__ cols,
                                  const int* __restrict__ int2full, const TE* __restrict__ elemK, TV* __restrict__ vals) {
    int R = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (R >= nfree) return;
    int fr = int2full[R];
    int ci = fr / ncp, Ar = fr - ci * ncp;
    int ir = Ar % n1, jr = Ar / n1;
    int NB1 = p + 1, D = 3 * NB1 * NB1;
    for (int z = rowptr[R] + lane; z < rowptr[R + 1]; z += 32) {
        int fc = int2full[cols[z]];
        int cj = fc / ncp, Ac = fc - cj * ncp;
        int ic = Ac % n1, jc = Ac / n1;
        int e1lo = max(max(ir, ic) - p, 0), e1hi = min(min(ir, ic), m1 - 1);
        int e2lo = max(max(jr, jc) - p, 0), e2hi = min(min(jr, jc), m2 - 1);
        double s = 0.0;
        for (int e2 = e2lo; e2 <= e2hi; ++e2)
            for (int e1 = e1lo; e1 <= e1hi; ++e1) {
                int la = (jr - e2) * NB1 + (ir - e1), lb = (jc - e2) * NB1 + (ic - e1);
                s += (double)elemK[((size_t)(e2 * m1 + e1) * D + 3 * la + ci) * D + 3 * lb + cj];
            }
        vals[z] = (TV)s;
    }
}

__global__ void vec_gather_kernel(int nfree, int p, int n1, int m1, int m2, int ncp, const int* __restrict__ int2full,
                                  const double* __restrict__ elemR, double* __restrict__ out, double alpha = 0.0,
                                  const double* __restrict__ y = nullptr, const double* __restrict__ alpha_sub = nullptr) {
    int R = blockIdx.x * blockDim.x + threadIdx.x;
    if (R >= nfree) return;
    int fr = int2full[R];
    int ci = fr / ncp, A = fr - ci * ncp;
    int i = A % n1, j = A / n1;
    int NB1 = p + 1, D = 3 * NB1 * NB1;
    double s = 0.0;
    for (int e2 = max(j - p, 0); e2 <= min(j, m2 - 1); ++e2)
        for (int e1 = max(i - p, 0); e1 <= min(i, m1 - 1); ++e1) {
            int la = (j - e2) * NB1 + (i - e1);
            s += elemR[(size_t)(e2 * m1 + e1) * D + 3 * la + ci];
        }
    if (y) {
        const double a = alpha_sub ? alpha - *alpha_sub : alpha;
        s += a * y[R];
    }
    out[R] = s;
}

__global__ void scatter_free_kernel(int nfree, const int* __restrict__ int2full, const double* __restrict__ x,
                                    double* __restrict__ ufull) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nfree) ufull[int2full[r]] = x[r];
}

__global__ void scatter_sum_kernel(int nfree, const int* __restrict__ int2full, const double* __restrict__ a,
                                   const double* __restrict__ b, double* __restrict__ x, double* __restrict__ ufull) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nfree) return;
    const double v = a[r] + b[r];
    x[r] = v;
    ufull[int2full[r]] = v;
}

__global__ void permute_kernel(int n, int nv, const int* __restrict__ map, const double* __restrict__ src,
                               double* __restrict__ dst) {
    // dst[map[i]] = src[i]
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int v = 0; v < nv; ++v) dst[(size_t)v * n + map[i]] = src[(size_t)v * n + i];
}

template <class TV>
__global__ void spmv_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ cols,
                            const TV* __restrict__ vals, const double* __restrict__ x, double* __restrict__ y) {
    // one warp per row
    int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;
    double s = 0.0;
    for (int k = rowptr[row] + lane; k < rowptr[row + 1]; k += 32) s += (double)vals[k] * x[cols[k]];
    s = warp_sum(s);
    if (lane == 0) y[row] = s;
}

// Batched CSR gather (FP32 values): one warp per row of the merged block-diagonal matrix; the
// instance of the row by binary search over the row offsets.
__global__ void csr_gather_batch_kernel(int nrows, int ninst, const int* __restrict__ dof_off,
                                        const BatchInst* __restrict__ desc, const int* __restrict__ rowptr,
                                        const int* __restrict__ cols, float* __restrict__ vals) {
    int R = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    int lane = threadIdx.x & 31;
    if (R >= nrows) return;
    const BatchInst& d = desc[find_segment(dof_off, ninst, R)];
    const int p = d.p, n1 = d.n1, m1 = d.m1, m2 = d.m2, ncp = d.ncp, off = d.dof_off;
    int fr = d.int2full[R - off];
    int ci = fr / ncp, Ar = fr - ci * ncp;
    int ir = Ar % n1, jr = Ar / n1;
    int NB1 = p + 1, D = 3 * NB1 * NB1;
    for (int z = rowptr[R] + lane; z < rowptr[R + 1]; z += 32) {
        int fc = d.int2full[cols[z] - off];
        int cj = fc / ncp, Ac = fc - cj * ncp;
        int ic = Ac % n1, jc = Ac / n1;
        int e1lo = max(max(ir, ic) - p, 0), e1hi = min(min(ir, ic), m1 - 1);
        int e2lo = max(max(jr, jc) - p, 0), e2hi = min(min(jr, jc), m2 - 1);
        double sum = 0.0;
        for (int e2 = e2lo; e2 <= e2hi; ++e2)
            for (int e1 = e1lo; e1 <= e1hi; ++e1) {
                int la = (jr - e2) * NB1 + (ir - e1), lb = (jc - e2) * NB1 + (ic - e1);
                sum += (double)d.elemK[((size_t)(e2 * m1 + e1) * D + 3 * la + ci) * D + 3 * lb + cj];
            }
        vals[z] = (float)sum;
    }
}

__global__ void vec_gather_batch_kernel(int nrows, int ninst, const int* __restrict__ dof_off,
                                        const BatchInst* __restrict__ desc, double* __restrict__ out) {
    int R = blockIdx.x * blockDim.x + threadIdx.x;
    if (R >= nrows) return;
    const BatchInst& d = desc[find_segment(dof_off, ninst, R)];
    const int p = d.p, n1 = d.n1, m1 = d.m1, m2 = d.m2, ncp = d.ncp;
    int fr = d.int2full[R - d.dof_off];
    int ci = fr / ncp, A = fr - ci * ncp;
    int i = A % n1, j = A / n1;
    int NB1 = p + 1, D = 3 * NB1 * NB1;
    double sum = 0.0;
    for (int e2 = max(j - p, 0); e2 <= min(j, m2 - 1); ++e2)
        for (int e1 = max(i - p, 0); e1 <= min(i, m1 - 1); ++e1) {
            int la = (j - e2) * NB1 + (i - e1);
            sum += d.elemR[(size_t)(e2 * m1 + e1) * D + 3 * la + ci];
        }
    out[R] = sum;
}

__global__ void scatter_free_batch_kernel(int nrows, int ninst, const int* __restrict__ dof_off,
                                          const BatchInst* __restrict__ desc, const double* __restrict__ x) {
    int R = blockIdx.x * blockDim.x + threadIdx.x;
    if (R >= nrows) return;
    const BatchInst& d = desc[find_segment(dof_off, ninst, R)];
    d.ufull[d.int2full[R - d.dof_off]] = x[R];
}

bool g_pairs_ready = false;

void init_pairs() {
    if (g_pairs_ready) return;
    unsigned char A[4][325] = {}, B[4][325] = {};
    for (int P = 1; P <= 4; ++P) {
        int nb = (P + 1) * (P + 1), k = 0;
        for (int a = 0; a < nb; ++a)
            for (int b = a; b < nb; ++b) { A[P - 1][k] = (unsigned char)a; B[P - 1][k] = (unsigned char)b; ++k; }
    }
    KL_CUDA(cudaMemcpyToSymbol(c_pairA, A, sizeof(A)));
    KL_CUDA(cudaMemcpyToSymbol(c_pairB, B, sizeof(B)));
    g_pairs_ready = true;
}

template <class T>
void launch_tangent(Problem& P, T* elemK) {
    init_pairs();
    int grid = ceil_div(P.nel, 4);
    double tm = P.t, tb = P.t * P.t * P.t / 12.0;
    switch (P.p) {
        case 2: kl_tangent_kernel<2, T><<<grid, 128, 0, P.stream>>>(P.nel, P.m1, P.n1, P.ncp, P.nq, P.d_tab1.get(), P.d_tab2.get(), P.d_qpgeo.get(), P.d_ufull.get(), tm, tb, elemK); break;
        case 3: kl_tangent_kernel<3, T><<<grid, 128, 0, P.stream>>>(P.nel, P.m1, P.n1, P.ncp, P.nq, P.d_tab1.get(), P.d_tab2.get(), P.d_qpgeo.get(), P.d_ufull.get(), tm, tb, elemK); break;
        default: throw std::invalid_argument("unsupported degree");
    }
    count_launch();
    KL_CHECK_LAUNCH();
}

}  // namespace

void Problem::set_displacement(const double* d_x) {
    scatter_free_kernel<<<ceil_div(nfree, 256), 256, 0, stream>>>(nfree, d_int2full.get(), d_x, d_ufull.get());
    count_launch();
    KL_CHECK_LAUNCH();
}

void Problem::set_displacement_sum(const double* a, const double* b, double* x) {
    scatter_sum_kernel<<<ceil_div(nfree, 256), 256, 0, stream>>>(nfree, d_int2full.get(), a, b, x, d_ufull.get());
    count_launch();
    KL_CHECK_LAUNCH();
}

void Problem::tangent_f32() {
    int D = 3 * (p + 1) * (p + 1);
    if (d_elemKf.size() < (size_t)nel * D * D) d_elemKf.alloc((size_t)nel * D * D);
    if (d_vals32.size() < (size_t)nnz) d_vals32.alloc(nnz);
    launch_tangent<float>(*this, d_elemKf.get());
    csr_gather_kernel<float, float><<<ceil_div((int64_t)nfree * 32, 256), 256, 0, stream>>>(nfree, nnz, p, n1, m1, m2, ncp, d_rowptr.get(), d_cols.get(), d_int2full.get(), d_elemKf.get(), d_vals32.get());
    count_launch();
    KL_CHECK_LAUNCH();
}

void Problem::tangent_f64() {
    int D = 3 * (p + 1) * (p + 1);
    if (d_elemKd.size() < (size_t)nel * D * D) d_elemKd.alloc((size_t)nel * D * D);
    if (d_vals64.size() < (size_t)nnz) d_vals64.alloc(nnz);
    launch_tangent<double>(*this, d_elemKd.get());
    csr_gather_kernel<double, double><<<ceil_div((int64_t)nfree * 32, 256), 256, 0, stream>>>(nfree, nnz, p, n1, m1, m2, ncp, d_rowptr.get(), d_cols.get(), d_int2full.get(), d_elemKd.get(), d_vals64.get());
    count_launch();
    KL_CHECK_LAUNCH();
}

void Problem::mass_f64() {
    init_pairs();
    int D = 3 * (p + 1) * (p + 1);
    if (d_elemKd.size() < (size_t)nel * D * D) d_elemKd.alloc((size_t)nel * D * D);
    if (d_vals64.size() < (size_t)nnz) d_vals64.alloc(nnz);
    int grid = ceil_div(nel, 4);
    double rt = rho * t;
    switch (p) {
        case 2: kl_mass_kernel<2><<<grid, 128, 0, stream>>>(nel, m1, nq, d_tab1.get(), d_tab2.get(), d_qpgeo.get(), rt, d_elemKd.get()); break;
        case 3: kl_mass_kernel<3><<<grid, 128, 0, stream>>>(nel, m1, nq, d_tab1.get(), d_tab2.get(), d_qpgeo.get(), rt, d_elemKd.get()); break;
        default: throw std::invalid_argument("unsupported degree");
    }
    count_launch();
    csr_gather_kernel<double, double><<<ceil_div((int64_t)nfree * 32, 256), 256, 0, stream>>>(nfree, nnz, p, n1, m1, m2, ncp, d_rowptr.get(), d_cols.get(), d_int2full.get(), d_elemKd.get(), d_vals64.get());
    count_launch();
    KL_CHECK_LAUNCH();
}

void Problem::internal_force(double* d_out, double alpha, const double* y, const double* alpha_sub) {
    int D = 3 * (p + 1) * (p + 1);
    if (d_elemR.size() < (size_t)nel * D) d_elemR.alloc((size_t)nel * D);
    int lpe = std::max((p + 1) * (p + 1), nq * nq);
    if (lpe > 32) throw std::invalid_argument("internal force kernel: (p+1)^2 and nq^2 must be <= 32");
    int es = 32 / lpe;
    int grid = ceil_div(nel, 4 * es);
    double tm = t, tb = t * t * t / 12.0;
    switch (p) {
        case 2:
            if (fint_fp64) kl_fint_kernel<2><<<grid, 128, 0, stream>>>(nel, m1, n1, ncp, nq, d_tab1.get(), d_tab2.get(), d_qpgeo.get(), d_ufull.get(), tm, tb, d_elemR.get());
            else kl_fint_df_kernel<2><<<grid, 128, 0, stream>>>(nel, m1, n1, ncp, nq, d_tab1.get(), d_tab2.get(), d_tab1s.get(), d_tab2s.get(), d_qpgeo.get(), d_ufull.get(), tm, tb, d_elemR.get());
            break;
        case 3:
            if (fint_fp64) kl_fint_kernel<3><<<grid, 128, 0, stream>>>(nel, m1, n1, ncp, nq, d_tab1.get(), d_tab2.get(), d_qpgeo.get(), d_ufull.get(), tm, tb, d_elemR.get());
            else kl_fint_df_kernel<3><<<grid, 128, 0, stream>>>(nel, m1, n1, ncp, nq, d_tab1.get(), d_tab2.get(), d_tab1s.get(), d_tab2s.get(), d_qpgeo.get(), d_ufull.get(), tm, tb, d_elemR.get());
            break;
        default: throw std::invalid_argument("unsupported degree");
    }
    count_launch();
    vec_gather_kernel<<<ceil_div(nfree, 256), 256, 0, stream>>>(nfree, p, n1, m1, m2, ncp, d_int2full.get(), d_elemR.get(), d_out,
                                                                alpha, y, alpha_sub);
    count_launch();
    KL_CHECK_LAUNCH();
}

void Problem::internal_force_elements(double* elemR) {
    int lpe = std::max((p + 1) * (p + 1), nq * nq);
    if (lpe > 32) throw std::invalid_argument("internal force kernel: (p+1)^2 and nq^2 must be <= 32");
    int grid = ceil_div(nel, 4 * (32 / lpe));
    double tm = t, tb = t * t * t / 12.0;
    switch (p) {
        case 2:
            if (fint_fp64) kl_fint_kernel<2><<<grid, 128, 0, stream>>>(nel, m1, n1, ncp, nq, d_tab1.get(), d_tab2.get(), d_qpgeo.get(), d_ufull.get(), tm, tb, elemR);
            else kl_fint_df_kernel<2><<<grid, 128, 0, stream>>>(nel, m1, n1, ncp, nq, d_tab1.get(), d_tab2.get(), d_tab1s.get(), d_tab2s.get(), d_qpgeo.get(), d_ufull.get(), tm, tb, elemR);
            break;
        case 3:
            if (fint_fp64) kl_fint_kernel<3><<<grid, 128, 0, stream>>>(nel, m1, n1, ncp, nq, d_tab1.get(), d_tab2.get(), d_qpgeo.get(), d_ufull.get(), tm, tb, elemR);
            else kl_fint_df_kernel<3><<<grid, 128, 0, stream>>>(nel, m1, n1, ncp, nq, d_tab1.get(), d_tab2.get(), d_tab1s.get(), d_tab2s.get(), d_qpgeo.get(), d_ufull.get(), tm, tb, elemR);
            break;
        default: throw std::invalid_argument("unsupported degree");
    }
    count_launch();
}

// ---- batched launches --------------------------------------------------------------------
void BatchedProblem::launch_tangent(int d, int bps) {
    DegreeList& L = deg[d];
    if (L.ninst == 0) return;
    init_pairs();
    int grid = std::max(1, std::min(ceil_div(L.nel, 4), num_sms * bps));
    if (d == 0)
        kl_tangent_batch_kernel<2><<<grid, 128, 0, stream>>>(L.ninst, L.insts.get(), L.elem_off.get(), d_desc.get());
    else
        kl_tangent_batch_kernel<3><<<grid, 128, 0, stream>>>(L.ninst, L.insts.get(), L.elem_off.get(), d_desc.get());
    count_launch();
    KL_CHECK_LAUNCH();
}

void BatchedProblem::launch_gather_K() {
    csr_gather_batch_kernel<<<ceil_div((int64_t)nfree * 32, 256), 256, 0, stream>>>(
        nfree, ninst, d_dof_off.get(), d_desc.get(), d_rowptr.get(), d_cols.get(), d_vals32.get());
    count_launch();
    KL_CHECK_LAUNCH();
}

void BatchedProblem::launch_fint(int d, int bps) {
    DegreeList& L = deg[d];
    if (L.ninst == 0) return;
    int grid = std::max(1, std::min(ceil_div(L.ngrp, 4), num_sms * bps));
    if (d == 0)
        kl_fint_batch_kernel<2><<<grid, 128, 0, stream>>>(L.ninst, L.insts.get(), L.grp_off.get(), d_desc.get());
    else
        kl_fint_batch_kernel<3><<<grid, 128, 0, stream>>>(L.ninst, L.insts.get(), L.grp_off.get(), d_desc.get());
    count_launch();
    KL_CHECK_LAUNCH();
}

void BatchedProblem::launch_gather_R(double* d_out) {
    vec_gather_batch_kernel<<<ceil_div(nfree, 256), 256, 0, stream>>>(nfree, ninst, d_dof_off.get(), d_desc.get(),
                                                                     d_out);
    count_launch();
    KL_CHECK_LAUNCH();
}

void BatchedProblem::set_displacement(const double* d_x) {
    scatter_free_batch_kernel<<<ceil_div(nfree, 256), 256, 0, stream>>>(nfree, ninst, d_dof_off.get(), d_desc.get(),
                                                                       d_x);
    count_launch();
    KL_CHECK_LAUNCH();
}

void BatchedProblem::tangent_f32() {
    launch_tangent(0, tangent_bps[0]);
    launch_tangent(1, tangent_bps[1]);
    launch_gather_K();
}

void BatchedProblem::internal_force(double* d_out) {
    launch_fint(0, fint_bps[0]);
    launch_fint(1, fint_bps[1]);
    launch_gather_R(d_out);
}

void Problem::pub_to_int(const double* d_pub, double* d_int, int nv) {
    permute_kernel<<<ceil_div(nfree, 256), 256, 0, stream>>>(nfree, nv, d_pub2int.get(), d_pub, d_int);
    count_launch();
    KL_CHECK_LAUNCH();
}

void Problem::int_to_pub(const double* d_int, double* d_pub, int nv) {
    permute_kernel<<<ceil_div(nfree, 256), 256, 0, stream>>>(nfree, nv, d_int2pub.get(), d_int, d_pub);
    count_launch();
    KL_CHECK_LAUNCH();
}

void Problem::upload_pub(const double* h_pub, double* d_int, int nv) {
    if (d_tmp_pub.size() < (size_t)nfree * nv) d_tmp_pub.alloc((size_t)nfree * nv);
    KL_CUDA(cudaMemcpyAsync(d_tmp_pub.get(), h_pub, sizeof(double) * nfree * nv, cudaMemcpyHostToDevice, stream));
    pub_to_int(d_tmp_pub.get(), d_int, nv);
}

void Problem::download_pub(const double* d_int, double* h_pub, int nv) {
    if (d_tmp_pub.size() < (size_t)nfree * nv) d_tmp_pub.alloc((size_t)nfree * nv);
    int_to_pub(d_int, d_tmp_pub.get(), nv);
    KL_CUDA(cudaMemcpyAsync(h_pub, d_tmp_pub.get(), sizeof(double) * nfree * nv, cudaMemcpyDeviceToHost, stream));
    KL_CUDA(cudaStreamSynchronize(stream));
}

void Problem::csr_to_host_pub(bool f64, int64_t* rowptr_out, int32_t* cols_out, double* vals_out) {
    // download internal-order values, then re-index rows/cols to the public order on the host
    std::vector<double> v(nnz);
    if (f64) {
        KL_CUDA(cudaMemcpyAsync(v.data(), d_vals64.get(), sizeof(double) * nnz, cudaMemcpyDeviceToHost, stream));
        KL_CUDA(cudaStreamSynchronize(stream));
    } else {
        std::vector<float> vf(nnz);
        KL_CUDA(cudaMemcpyAsync(vf.data(), d_vals32.get(), sizeof(float) * nnz, cudaMemcpyDeviceToHost, stream));
        KL_CUDA(cudaStreamSynchronize(stream));
        for (int64_t z = 0; z < nnz; ++z) v[z] = vf[z];
    }
    rowptr_out[0] = 0;
    for (int pr = 0; pr < nfree; ++pr) {
        int R = pub2int[pr];
        rowptr_out[pr + 1] = rowptr_out[pr] + (rowptr[R + 1] - rowptr[R]);
    }
    std::vector<std::pair<int, double>> row;
    for (int pr = 0; pr < nfree; ++pr) {
        int R = pub2int[pr];
        row.clear();
        for (int z = rowptr[R]; z < rowptr[R + 1]; ++z) row.emplace_back(int2pub[cols[z]], v[z]);
        std::sort(row.begin(), row.end());
        int64_t o = rowptr_out[pr];
        for (size_t k = 0; k < row.size(); ++k) { cols_out[o + k] = row[k].first; vals_out[o + k] = row[k].second; }
    }
}

void spmv(const Problem& P, bool f64, const double* x, double* y) {
    if ((f64 ? P.d_vals64.size() : P.d_vals32.size()) < (size_t)P.nnz)
        throw std::logic_error("spmv: matrix values not assembled");
    int grid = ceil_div((int64_t)P.nfree * 32, 256);
    if (f64) spmv_kernel<double><<<grid, 256, 0, P.stream>>>(P.nfree, P.d_rowptr.get(), P.d_cols.get(), P.d_vals64.get(), x, y);
    else spmv_kernel<float><<<grid, 256, 0, P.stream>>>(P.nfree, P.d_rowptr.get(), P.d_cols.get(), P.d_vals32.get(), x, y);
    count_launch();
    KL_CHECK_LAUNCH();
}

}  // namespace klsa
