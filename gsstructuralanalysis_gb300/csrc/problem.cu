// problem.cu -- host set-up of a patch problem: B-spline tables, Gauss-point geometry,
// dof maps, nested-dissection numbering, CSR pattern, external loads.
#include <cstdlib>
#include "problem.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>

#include "../../include/klshell_gb300.h"

namespace klsa {

std::atomic<unsigned long long> g_launch_count{0};
thread_local unsigned long long* t_capture_count = nullptr;
PhaseTimer g_timer;

namespace {

constexpr int MAXP = 4;

// Gauss-Legendre rule on [-1, 1] (Newton iteration on the three-term recurrence).
void gauss_rule(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int i = 0; i < (n + 1) / 2; ++i) {
        double z = std::cos(M_PI * (4.0 * i + 3.0) / (4.0 * n + 2.0));
        double dp = 1.0;
        for (int it = 0; it < 60; ++it) {
            double pm1 = 1.0, pc = z;
            for (int kk = 2; kk <= n; ++kk) {
                double pn = ((2.0 * kk - 1.0) * z * pc - (kk - 1.0) * pm1) / kk;
                pm1 = pc;
                pc = pn;
            }
            if (n == 1) { pc = z; pm1 = 1.0; }
            dp = n * (pm1 - z * pc) / (1.0 - z * z);
            double dz = pc / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-15) break;
        }
        x[i] = -z;
        x[n - 1 - i] = z;
        w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

// Nonzero B-spline functions of degree p at u on knot span `span` and their derivatives up to
// order 2: ders[d*(p+1) + a] for function span-p+a.  Triangular table of the lower-degree
// functions and knot differences; derivatives from the differences of that table.
void bspline_ders(int span, double u, int p, const double* U, double* ders) {
    double ndu[MAXP + 1][MAXP + 1];   // ndu[j][r]: functions (upper incl. diag), knot diffs (lower)
    double left[MAXP + 1], right[MAXP + 1];
    ndu[0][0] = 1.0;
    for (int j = 1; j <= p; ++j) {
        left[j] = u - U[span + 1 - j];
        right[j] = U[span + j] - u;
        double saved = 0.0;
        for (int r = 0; r < j; ++r) {
            ndu[j][r] = right[r + 1] + left[j - r];
            double tmp = ndu[r][j - 1] / ndu[j][r];
            ndu[r][j] = saved + right[r + 1] * tmp;
            saved = left[j - r] * tmp;
        }
        ndu[j][j] = saved;
    }
    for (int a = 0; a <= p; ++a) ders[a] = ndu[a][p];
    double coef[2][MAXP + 1];
    for (int r = 0; r <= p; ++r) {
        int s1 = 0, s2 = 1;
        coef[0][0] = 1.0;
        for (int kd = 1; kd <= 2; ++kd) {
            double dsum = 0.0;
            int rk = r - kd, pk = p - kd;
            if (kd > p) { ders[kd * (p + 1) + r] = 0.0; continue; }
            if (r >= kd) {
                coef[s2][0] = coef[s1][0] / ndu[pk + 1][rk];
                dsum = coef[s2][0] * ndu[rk][pk];
            }
            int j1 = (rk >= -1) ? 1 : -rk;
            int j2 = (r - 1 <= pk) ? kd - 1 : p - r;
            for (int j = j1; j <= j2; ++j) {
                coef[s2][j] = (coef[s1][j] - coef[s1][j - 1]) / ndu[pk + 1][rk + j];
                dsum += coef[s2][j] * ndu[rk + j][pk];
            }
            if (r <= pk) {
                coef[s2][kd] = -coef[s1][kd - 1] / ndu[pk + 1][r];
                dsum += coef[s2][kd] * ndu[r][pk];
            }
            ders[kd * (p + 1) + r] = dsum;
            std::swap(s1, s2);
        }
    }
    for (int a = 0; a <= p; ++a) {
        ders[1 * (p + 1) + a] *= p;
        ders[2 * (p + 1) + a] *= (p >= 2) ? p * (p - 1) : 0.0;
    }
}

int span_of(int ncp, int p, double u, const double* U) {
    if (u >= U[ncp]) return ncp - 1;
    int s = (int)(std::upper_bound(U + p, U + ncp + 1, u) - U) - 1;
    return std::max(p, std::min(s, ncp - 1));
}

struct V3 { double x, y, z; };
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scl(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dt(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cr(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

void check_knots(const std::vector<double>& U, int n, int p) {
    if ((int)U.size() != n + p + 1) throw std::invalid_argument("knot vector length must be n+p+1");
    for (int i = 0; i < p; ++i)
        if (U[i] != U[i + 1] || U[n + p - i] != U[n + p - i - 1])
            throw std::invalid_argument("knot vectors must be open (p+1 repeated end knots)");
    for (int i = p; i < n; ++i)
        if (!(U[i + 1] > U[i])) throw std::invalid_argument("interior knots must be simple and increasing");
}

}  // namespace

Problem::Problem(const klsa_patch_desc& d) {
    p = d.p; n1 = d.n1; n2 = d.n2;
    nq = d.nq > 0 ? d.nq : d.p + 1;
    if (p < 2 || p > 3) throw std::invalid_argument("degree must be 2 or 3 (Kirchhoff-Love shells need C1 bases)");
    if (n1 <= p || n2 <= p) throw std::invalid_argument("need at least p+1 control points per direction");
    if (nq < 1 || nq > 8) throw std::invalid_argument("Gauss points per direction must be in 1..8");
    if (!d.knots1 || !d.knots2 || !d.ctrl || !d.fixed) throw std::invalid_argument("null description array");
    ncp = n1 * n2;
    m1 = n1 - p; m2 = n2 - p;
    nel = m1 * m2;
    nqp = nel * nq * nq;
    E = d.E; nu = d.nu; t = d.thickness; rho = d.density;
    U1.assign(d.knots1, d.knots1 + n1 + p + 1);
    U2.assign(d.knots2, d.knots2 + n2 + p + 1);
    check_knots(U1, n1, p);
    check_knots(U2, n2, p);
    X.assign(d.ctrl, d.ctrl + 3 * (size_t)ncp);
    fixed.assign(d.fixed, d.fixed + 3 * (size_t)ncp);

    // ---- 1-D tables and Gauss-point geometry (FP64) -----------------------------------
    std::vector<double> gx, gw;
    gauss_rule(nq, gx, gw);
    const int nb1 = p + 1;
    std::vector<double> tab1((size_t)m1 * nq * 3 * nb1), tab2((size_t)m2 * nq * 3 * nb1);
    std::vector<double> jw1((size_t)m1 * nq), jw2((size_t)m2 * nq);
    auto fill = [&](const std::vector<double>& U, int n, int m, std::vector<double>& tab, std::vector<double>& jw) {
        for (int e = 0; e < m; ++e) {
            double a = U[p + e], b = U[p + e + 1];
            for (int q = 0; q < nq; ++q) {
                double u = 0.5 * (a + b) + 0.5 * (b - a) * gx[q];
                double der[3 * (MAXP + 1)];
                int sp = span_of(n, p, u, U.data());
                if (sp != p + e) throw std::logic_error("span mismatch");
                bspline_ders(sp, u, p, U.data(), der);
                for (int k = 0; k < 3; ++k)
                    for (int aa = 0; aa < nb1; ++aa) tab[(((size_t)e * nq + q) * 3 + k) * nb1 + aa] = der[k * nb1 + aa];
                jw[(size_t)e * nq + q] = 0.5 * (b - a) * gw[q];
            }
        }
    };
    fill(U1, n1, m1, tab1, jw1);
    fill(U2, n2, m2, tab2, jw2);

    std::vector<double> qpgeo((size_t)nqp * QGEO);
    std::vector<double> F_full(3 * (size_t)ncp, 0.0);
    const double lam = E * nu / (1.0 - nu * nu), mu = E / (2.0 * (1.0 + nu));
    const bool has_surf = d.surface_load &&
                          (d.surface_load[0] != 0 || d.surface_load[1] != 0 || d.surface_load[2] != 0);
    for (int e2 = 0; e2 < m2; ++e2)
        for (int e1 = 0; e1 < m1; ++e1) {
            int e = e2 * m1 + e1;
            for (int q2 = 0; q2 < nq; ++q2)
                for (int q1 = 0; q1 < nq; ++q1) {
                    const double* t1 = &tab1[(((size_t)e1 * nq + q1) * 3) * nb1];
                    const double* t2 = &tab2[(((size_t)e2 * nq + q2) * 3) * nb1];
                    V3 A1{0, 0, 0}, A2{0, 0, 0}, X11{0, 0, 0}, X22{0, 0, 0}, X12{0, 0, 0};
                    for (int b = 0; b < nb1; ++b)
                        for (int a = 0; a < nb1; ++a) {
                            int A = (e2 + b) * n1 + (e1 + a);
                            V3 XA{X[3 * A], X[3 * A + 1], X[3 * A + 2]};
                            A1 = add(A1, scl(t1[nb1 + a] * t2[b], XA));
                            A2 = add(A2, scl(t1[a] * t2[nb1 + b], XA));
                            X11 = add(X11, scl(t1[2 * nb1 + a] * t2[b], XA));
                            X22 = add(X22, scl(t1[a] * t2[2 * nb1 + b], XA));
                            X12 = add(X12, scl(t1[nb1 + a] * t2[nb1 + b], XA));
                        }
                    double g11 = dt(A1, A1), g22 = dt(A2, A2), g12 = dt(A1, A2);
                    double det = g11 * g22 - g12 * g12;
                    double h11 = g22 / det, h22 = g11 / det, h12 = -g12 / det;   // contravariant metric
                    double dA = std::sqrt(dt(cr(A1, A2), cr(A1, A2))) * jw1[(size_t)e1 * nq + q1] * jw2[(size_t)e2 * nq + q2];
                    double* g = &qpgeo[((size_t)e * nq * nq + q2 * nq + q1) * QGEO];
                    V3 vv[5] = {A1, A2, X11, X22, X12};
                    for (int k = 0; k < 5; ++k) { g[3 * k] = vv[k].x; g[3 * k + 1] = vv[k].y; g[3 * k + 2] = vv[k].z; }
                    g[15] = (lam + 2 * mu) * h11 * h11;                // C^{1111}
                    g[16] = lam * h11 * h22 + 2 * mu * h12 * h12;      // C^{1122}
                    g[17] = (lam + 2 * mu) * h11 * h12;                // C^{1112}
                    g[18] = (lam + 2 * mu) * h22 * h22;                // C^{2222}
                    g[19] = (lam + 2 * mu) * h22 * h12;                // C^{2212}
                    g[20] = lam * h12 * h12 + mu * (h11 * h22 + h12 * h12);   // C^{1212}
                    g[21] = dA;
                    const V3 At = cr(A1, A2);
                    const double J0 = std::sqrt(dt(At, At));
                    const V3 A3{At.x / J0, At.y / J0, At.z / J0};
                    g[22] = dt(X11, A3);
                    g[23] = dt(X22, A3);
                    g[24] = dt(X12, A3);
                    if (has_surf)
                        for (int b = 0; b < nb1; ++b)
                            for (int a = 0; a < nb1; ++a) {
                                int A = (e2 + b) * n1 + (e1 + a);
                                double Nv = t1[a] * t2[b] * dA;
                                for (int c = 0; c < 3; ++c) F_full[(size_t)c * ncp + A] += Nv * d.surface_load[c];
                            }
                }
        }
    // point loads
    for (int kp = 0; kp < d.n_point_loads; ++kp) {
        const double* L = d.point_loads + 5 * kp;
        double b1[3 * (MAXP + 1)], b2[3 * (MAXP + 1)];
        int s1 = span_of(n1, p, L[0], U1.data()), s2 = span_of(n2, p, L[1], U2.data());
        bspline_ders(s1, L[0], p, U1.data(), b1);
        bspline_ders(s2, L[1], p, U2.data(), b2);
        for (int b = 0; b < nb1; ++b)
            for (int a = 0; a < nb1; ++a) {
                int A = (s2 - p + b) * n1 + (s1 - p + a);
                for (int c = 0; c < 3; ++c) F_full[(size_t)c * ncp + A] += b1[a] * b2[b] * L[2 + c];
            }
    }
    // edge line loads (per unit reference length)
    for (int ke = 0; ke < d.n_edge_loads; ++ke) {
        const double* L = d.edge_loads + 4 * ke;
        int side = (int)L[0];
        if (side < 0 || side > 3) throw std::invalid_argument("edge load side must be 0..3");
        bool along1 = side >= 2;
        double fixed_par = (side == 0 || side == 2) ? 0.0 : 1.0;
        int m = along1 ? m1 : m2;
        const std::vector<double>& Ue = along1 ? U1 : U2;
        for (int e = 0; e < m; ++e) {
            double a = Ue[p + e], b = Ue[p + e + 1];
            for (int q = 0; q < nq; ++q) {
                double s = 0.5 * (a + b) + 0.5 * (b - a) * gx[q];
                double xi1 = along1 ? s : fixed_par, xi2 = along1 ? fixed_par : s;
                double b1[3 * (MAXP + 1)], b2[3 * (MAXP + 1)];
                int s1 = span_of(n1, p, xi1, U1.data()), s2 = span_of(n2, p, xi2, U2.data());
                bspline_ders(s1, xi1, p, U1.data(), b1);
                bspline_ders(s2, xi2, p, U2.data(), b2);
                V3 T{0, 0, 0};
                for (int bb = 0; bb < nb1; ++bb)
                    for (int aa = 0; aa < nb1; ++aa) {
                        int A = (s2 - p + bb) * n1 + (s1 - p + aa);
                        double dN = along1 ? b1[nb1 + aa] * b2[bb] : b1[aa] * b2[nb1 + bb];
                        T = add(T, scl(dN, V3{X[3 * A], X[3 * A + 1], X[3 * A + 2]}));
                    }
                double ds = std::sqrt(dt(T, T)) * 0.5 * (b - a) * gw[q];
                for (int bb = 0; bb < nb1; ++bb)
                    for (int aa = 0; aa < nb1; ++aa) {
                        int A = (s2 - p + bb) * n1 + (s1 - p + aa);
                        double Nv = b1[aa] * b2[bb] * ds;
                        for (int c = 0; c < 3; ++c) F_full[(size_t)c * ncp + A] += Nv * L[1 + c];
                    }
            }
        }
    }

    // ---- nested dissection numbering and CSR pattern (internal order) ----------------
    tree = build_nd_tree(n1, n2, p, fixed.data(), 8);
    nfree = tree.nfree;
    if (nfree == 0) throw std::invalid_argument("no free degrees of freedom");
    rowptr.assign(nfree + 1, 0);
    {
        std::vector<std::vector<int>> cpcols(ncp);
        // columns of every row of control point A: free dofs of all cps within distance p
        int64_t total = 0;
        std::vector<int> rowcount(nfree, 0);
        for (int A = 0; A < ncp; ++A) {
            int i = A % n1, j = A / n1;
            bool any = false;
            for (int c = 0; c < 3; ++c) any |= tree.full2int[(size_t)c * ncp + A] >= 0;
            if (!any) continue;
            std::vector<int>& cl = cpcols[A];
            for (int j2 = std::max(0, j - p); j2 <= std::min(n2 - 1, j + p); ++j2)
                for (int i2 = std::max(0, i - p); i2 <= std::min(n1 - 1, i + p); ++i2)
                    for (int c = 0; c < 3; ++c) {
                        int id = tree.full2int[(size_t)c * ncp + j2 * n1 + i2];
                        if (id >= 0) cl.push_back(id);
                    }
            std::sort(cl.begin(), cl.end());
            for (int c = 0; c < 3; ++c) {
                int id = tree.full2int[(size_t)c * ncp + A];
                if (id >= 0) { rowcount[id] = (int)cl.size(); total += (int64_t)cl.size(); }
            }
        }
        if (total >= (int64_t)1 << 31) throw std::invalid_argument("problem too large for int32 CSR");
        for (int r = 0; r < nfree; ++r) rowptr[r + 1] = rowptr[r] + rowcount[r];
        nnz = rowptr[nfree];
        cols.assign(nnz, 0);
        for (int r = 0; r < nfree; ++r) {
            int full = tree.int2full[r];
            int A = full % ncp;
            std::copy(cpcols[A].begin(), cpcols[A].end(), cols.begin() + rowptr[r]);
        }
    }
    // public order: component-blocked free dofs
    pub2int.assign(nfree, -1);
    int2pub.assign(nfree, -1);
    {
        int k = 0;
        for (size_t f = 0; f < 3 * (size_t)ncp; ++f)
            if (!fixed[f]) {
                int id = tree.full2int[f];
                pub2int[k] = id;
                int2pub[id] = k;
                ++k;
            }
    }
    F_int_order.assign(nfree, 0.0);
    for (int r = 0; r < nfree; ++r) F_int_order[r] = F_full[tree.int2full[r]];

    // ---- device upload ------------------------------------------------------------------
    KL_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    d_tab1.upload(tab1, stream);
    d_tab2.upload(tab2, stream);
    std::vector<float> t1f(tab1.begin(), tab1.end()), t2f(tab2.begin(), tab2.end());
    d_tab1f.upload(t1f, stream);
    d_tab2f.upload(t2f, stream);
    {
        auto split = [](const std::vector<double>& t) {
            std::vector<float2> o(t.size());
            for (size_t i = 0; i < t.size(); ++i) {
                const float h = (float)t[i];
                o[i] = make_float2(h, (float)(t[i] - (double)h));
            }
            return o;
        };
        d_tab1s.upload(split(tab1), stream);
        d_tab2s.upload(split(tab2), stream);
    }
    if (const char* e = std::getenv("KLSA_RESIDUAL_FP64")) fint_fp64 = e[0] == '1';
    d_qpgeo.upload(qpgeo, stream);
    d_int2full.upload(tree.int2full, stream);
    d_full2int.upload(tree.full2int, stream);
    d_pub2int.upload(pub2int, stream);
    d_int2pub.upload(int2pub, stream);
    d_rowptr.upload(rowptr, stream);
    d_cols.upload(cols, stream);
    d_F.upload(F_int_order, stream);
    d_ufull.alloc(3 * (size_t)ncp);
    d_ufull.zero(stream);
    d_tmp_pub.alloc((size_t)nfree * 4);
    d_tmp_int.alloc((size_t)nfree * 4);
    KL_CUDA(cudaStreamSynchronize(stream));
}

Problem::~Problem() {
    mf.reset();
    mf64.reset();
    if (stream) cudaStreamDestroy(stream);
}

Multifrontal& Problem::solver() {
    if (!mf) mf.reset(new Multifrontal(tree, rowptr, cols, stream));
    return *mf;
}

Multifrontal64& Problem::solver64() {
    if (!mf64) mf64.reset(new Multifrontal64(tree, rowptr, cols, stream));
    return *mf64;
}

double Problem::flops_tangent() const {
    // per Gauss point and (A<=B) control-point pair: 9 entries x (18 material + 1 membrane
    // + 2 normal-derivative + 3 rank + 3 normal-pair + 1 cross) FMAs = 252 FMAs (504 flop);
    // per control point set-up ~ 400 flop; per point geometry ~ 300 flop.
    double nb = (p + 1.0) * (p + 1.0);
    double pairs = nb * (nb + 1.0) / 2.0;
    return (double)nqp * (pairs * 504.0 + nb * 400.0 + 300.0);
}

}  // namespace klsa
