// kl_oracle.cpp -- FP64 CPU oracle for the Kirchhoff-Love shell hot path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
// calls this file; only tests/, the smoke check and the CPU-baseline leg of
// bench.py use it, and only as the checker or the timed CPU comparator.
//
// What it restates
//   The reference module (gsStructuralAnalysis) calls gsKLShell's
//   gsThinShellAssembler for K(u), R(u), M and F (call sites:
//   unittests/gsStaticSolver_test.cpp:230-253, tutorials/nonlinear_shell_static.cpp:120-136,
//   tutorials/nonlinear_shell_arcLength.cpp:123-142).  gsKLShell is not part of
//   the reference tree (it is a separate gismo module pulled at an unpinned
//   branch head by .github/workflows/ci.yml:32-36), so this oracle restates the
//   published formulation it implements: the isogeometric Kirchhoff-Love shell of
//   Kiendl et al. (2009) with a St. Venant-Kirchhoff material in the
//   contravariant reference metric, (p+1)x(p+1) Gauss-Legendre points per
//   element (filedata/options/solver_options.xml:11-12), B-spline basis by the
//   Cox-de Boor recursion.  Parity of the assembly against gsKLShell itself is
//   therefore unpinned; the restatement is pinned by finite differences
//   (K = dFint/du), patch tests and the closed-form plate answers the reference
//   prints beside its own results (examples/gsThinShell_Modal.cpp:333).
//
// Conventions (shared with the CUDA path through the problem description only)
//   * control points: index A = j*n1 + i, i along parameter 1, j along parameter 2
//   * FULL dof vector: component-blocked [x_0..x_{ncp-1}, y..., z...], the layout
//     of gsThinShellAssembler::fullSolutionVector (benchmarks/benchmark_Wrinkling.cpp:684-686)
//   * strains: eps = 1/2 (a_ab - A_ab), kappa = B_ab - b_ab, Voigt with engineering shear
//   * Fint_r = int (n . d eps/du_r + m . d kappa/du_r) dA  (reference area)
//   This file evaluates the second variation dof-pair by dof-pair with explicit
//   vector derivatives of the unit normal; the CUDA kernels use an algebraically
//   regrouped form, so the two are independent implementations.
//
// Build: oracle/Makefile (g++ -O2 -fopenmp -shared -fPIC).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int MAXP = 4;             // highest supported degree
constexpr int MAXB = MAXP + 1;      // nonzero basis functions per direction
constexpr int MAXD = 3 * MAXB * MAXB;

struct Vec3 { double x, y, z; };
inline Vec3 operator+(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec3 operator-(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3 operator*(double s, Vec3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3 cross(Vec3 a, Vec3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double comp(Vec3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline Vec3 unit(int i) { return {i == 0 ? 1.0 : 0.0, i == 1 ? 1.0 : 0.0, i == 2 ? 1.0 : 0.0}; }

// Gauss-Legendre nodes on [-1,1] by Newton iteration on P_n.
void gauss_legendre(int n, double* x, double* w) {
    for (int i = 0; i < n; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = 0.0;
            for (int k = 1; k <= n; ++k) {
                double p2 = p1; p1 = p0;
                p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
            }
            double dp = n * (z * p0 - p1) / (z * z - 1.0);
            double dz = p0 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = 0.0;
        for (int k = 1; k <= n; ++k) {
            double p2 = p1; p1 = p0;
            p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
        }
        double dp = n * (z * p0 - p1) / (z * z - 1.0);
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

int find_span(int ncp, int p, double u, const double* U) {
    if (u >= U[ncp]) return ncp - 1;
    if (u <= U[p]) return p;
    int lo = p, hi = ncp;
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (u < U[mid]) hi = mid; else lo = mid;
    }
    return lo;
}

// Cox-de Boor tables: tab[k][m] = N_{span-k+m, k}(u), k = 0..p, m = 0..k.
struct BasisTable {
    int span, p;
    const double* U;
    double tab[MAXP + 1][MAXB];
    double N(int i, int k) const {  // N_{i,k}(u)
        int m = i - (span - k);
        if (m < 0 || m > k) return 0.0;
        return tab[k][m];
    }
    // d-th derivative of N_{i,k} from lower-degree values (recursive, d <= 2)
    double der(int i, int k, int d) const {
        if (d == 0) return N(i, k);
        double a = U[i + k] - U[i], b = U[i + k + 1] - U[i + 1];
        double r = 0.0;
        if (a > 0) r += der(i, k - 1, d - 1) / a;
        if (b > 0) r -= der(i + 1, k - 1, d - 1) / b;
        return k * r;
    }
};

void basis_table(int span, double u, int p, const double* U, BasisTable& T) {
    T.span = span; T.p = p; T.U = U;
    T.tab[0][0] = 1.0;
    for (int k = 1; k <= p; ++k) {
        for (int m = 0; m <= k; ++m) {
            int i = span - k + m;
            double v = 0.0;
            // left term: (u - U_i)/(U_{i+k} - U_i) N_{i,k-1}
            {
                double den = U[i + k] - U[i];
                int mm = i - (span - (k - 1));
                if (den > 0 && mm >= 0 && mm <= k - 1) v += (u - U[i]) / den * T.tab[k - 1][mm];
            }
            // right term: (U_{i+k+1} - u)/(U_{i+k+1} - U_{i+1}) N_{i+1,k-1}
            {
                double den = U[i + k + 1] - U[i + 1];
                int mm = i + 1 - (span - (k - 1));
                if (den > 0 && mm >= 0 && mm <= k - 1) v += (U[i + k + 1] - u) / den * T.tab[k - 1][mm];
            }
            T.tab[k][m] = v;
        }
    }
}

// values/derivatives of the p+1 functions span-p..span at u: out[d][a]
void basis_ders(int ncp, int p, const double* U, double u, int& span, double out[3][MAXB]) {
    span = find_span(ncp, p, u, U);
    BasisTable T;
    basis_table(span, u, p, U, T);
    for (int a = 0; a <= p; ++a)
        for (int d = 0; d < 3; ++d) out[d][a] = (d <= p) ? T.der(span - p + a, p, d) : 0.0;
}

struct Patch {
    int p, n1, n2, nq;
    const double* U1;
    const double* U2;
    const double* X;   // ncp*3, cp-major (A*3+c)
    double E, nu, t, rho;
    const double* W = nullptr;   // NURBS weights (ncp); null: B-spline (all weights 1)
};

// Rational basis of a NURBS patch from the tensor-product B-spline values at one point:
// R_A = w_A N_A / W with W = sum_B w_B N_B, and by the quotient rule (o_a = W,a / W)
//   R_A,a  = (w_A / W) (N_A,a - N_A o_a)
//   R_A,ab = (w_A / W) (N_A,ab - N_A,a o_b - N_A,b o_a + N_A (2 o_a o_b - W,ab / W)).
// N, N1, N2, N11, N22, N12 (nb values each) are replaced in place; w holds the nb weights.
void rationalize(int nb, const double* w, double* N, double* N1, double* N2, double* N11, double* N22,
                 double* N12) {
    double W = 0, W1 = 0, W2 = 0, W11 = 0, W22 = 0, W12 = 0;
    for (int k = 0; k < nb; ++k) {
        W += w[k] * N[k];
        W1 += w[k] * N1[k];
        W2 += w[k] * N2[k];
        W11 += w[k] * N11[k];
        W22 += w[k] * N22[k];
        W12 += w[k] * N12[k];
    }
    const double iW = 1.0 / W, o1 = W1 * iW, o2 = W2 * iW;
    const double c11 = 2 * o1 * o1 - W11 * iW, c22 = 2 * o2 * o2 - W22 * iW, c12 = 2 * o1 * o2 - W12 * iW;
    for (int k = 0; k < nb; ++k) {
        const double c = w[k] * iW, n0 = N[k], n1 = N1[k], n2 = N2[k];
        N[k] = c * n0;
        N1[k] = c * (n1 - n0 * o1);
        N2[k] = c * (n2 - n0 * o2);
        N11[k] = c * (N11[k] - 2 * n1 * o1 + n0 * c11);
        N22[k] = c * (N22[k] - 2 * n2 * o2 + n0 * c22);
        N12[k] = c * (N12[k] - n1 * o2 - n2 * o1 + n0 * c12);
    }
}

struct Elem {
    int s1, s2;          // knot spans
    double u0, u1, v0, v1;
};

std::vector<Elem> elements(const Patch& P) {
    std::vector<Elem> els;
    for (int s2 = P.p; s2 < P.n2; ++s2) {
        if (!(P.U2[s2 + 1] > P.U2[s2])) continue;
        for (int s1 = P.p; s1 < P.n1; ++s1) {
            if (!(P.U1[s1 + 1] > P.U1[s1])) continue;
            els.push_back({s1, s2, P.U1[s1], P.U1[s1 + 1], P.U2[s2], P.U2[s2 + 1]});
        }
    }
    return els;
}

// Quantities of one quadrature point.
struct QP {
    int nb;                      // (p+1)^2
    int cp[MAXB * MAXB];         // global control point index
    double N[MAXB * MAXB], N1[MAXB * MAXB], N2[MAXB * MAXB];
    double N11[MAXB * MAXB], N22[MAXB * MAXB], N12[MAXB * MAXB];
    double dA;                   // |A1 x A2| * weight * parametric jacobian
};

void eval_qp(const Patch& P, const Elem& e, double xi1, double xi2, double wq, QP& q, Vec3& A1, Vec3& A2) {
    int sp1, sp2;
    double b1[3][MAXB], b2[3][MAXB];
    basis_ders(P.n1, P.p, P.U1, xi1, sp1, b1);
    basis_ders(P.n2, P.p, P.U2, xi2, sp2, b2);
    int nb1 = P.p + 1;
    q.nb = nb1 * nb1;
    A1 = {0, 0, 0}; A2 = {0, 0, 0};
    for (int b = 0; b < nb1; ++b)
        for (int a = 0; a < nb1; ++a) {
            int k = b * nb1 + a;
            int gi = sp1 - P.p + a, gj = sp2 - P.p + b;
            q.cp[k] = gj * P.n1 + gi;
            q.N[k] = b1[0][a] * b2[0][b];
            q.N1[k] = b1[1][a] * b2[0][b];
            q.N2[k] = b1[0][a] * b2[1][b];
            q.N11[k] = b1[2][a] * b2[0][b];
            q.N22[k] = b1[0][a] * b2[2][b];
            q.N12[k] = b1[1][a] * b2[1][b];
        }
    if (P.W) {
        double w[MAXB * MAXB];
        for (int k = 0; k < q.nb; ++k) w[k] = P.W[q.cp[k]];
        rationalize(q.nb, w, q.N, q.N1, q.N2, q.N11, q.N22, q.N12);
    }
    for (int k = 0; k < q.nb; ++k) {
        const double* Xa = P.X + 3 * q.cp[k];
        Vec3 XA{Xa[0], Xa[1], Xa[2]};
        A1 = A1 + q.N1[k] * XA;
        A2 = A2 + q.N2[k] * XA;
    }
    (void)e;
    q.dA = std::sqrt(dot(cross(A1, A2), cross(A1, A2))) * wq;
}

// SVK material matrix (Voigt, engineering shear) in the contravariant reference metric.
void material(const Patch& P, double A11, double A12, double A22, double C[3][3]) {
    double det = A11 * A22 - A12 * A12;
    double c11 = A22 / det, c22 = A11 / det, c12 = -A12 / det;   // contravariant A^{ab}
    double lam = P.E * P.nu / (1.0 - P.nu * P.nu);
    double mu = P.E / (2.0 * (1.0 + P.nu));
    C[0][0] = (lam + 2 * mu) * c11 * c11;
    C[1][1] = (lam + 2 * mu) * c22 * c22;
    C[0][1] = C[1][0] = lam * c11 * c22 + 2 * mu * c12 * c12;
    C[0][2] = C[2][0] = (lam + 2 * mu) * c11 * c12;
    C[1][2] = C[2][1] = (lam + 2 * mu) * c22 * c12;
    C[2][2] = lam * c12 * c12 + mu * (c11 * c22 + c12 * c12);
}

// One element: Ke (d x d, local dof r = 3*a + i) and Fint_e (d).
void element_kl(const Patch& P, const Elem& e, const double* ufull, int ncp, bool wantK,
                std::vector<double>& Ke, std::vector<double>& Fe, int& nb) {
    const int p = P.p, nq = P.nq;
    double gx[16], gw[16];
    gauss_legendre(nq, gx, gw);
    nb = (p + 1) * (p + 1);
    const int d = 3 * nb;
    Ke.assign(wantK ? d * d : 0, 0.0);
    Fe.assign(d, 0.0);
    double jac = 0.25 * (e.u1 - e.u0) * (e.v1 - e.v0);
    for (int q2 = 0; q2 < nq; ++q2)
        for (int q1 = 0; q1 < nq; ++q1) {
            double xi1 = 0.5 * (e.u0 + e.u1) + 0.5 * (e.u1 - e.u0) * gx[q1];
            double xi2 = 0.5 * (e.v0 + e.v1) + 0.5 * (e.v1 - e.v0) * gx[q2];
            QP q;
            Vec3 A1, A2;
            eval_qp(P, e, xi1, xi2, gw[q1] * gw[q2] * jac, q, A1, A2);
            // reference and deformed derivatives
            // reference derivatives from X, displacement derivatives from u (kept separate so that
            // small displacements are not lost in X + u)
            Vec3 X11{0, 0, 0}, X22{0, 0, 0}, X12{0, 0, 0};
            Vec3 d1{0, 0, 0}, d2{0, 0, 0}, d11{0, 0, 0}, d22{0, 0, 0}, d12{0, 0, 0};
            for (int k = 0; k < nb; ++k) {
                int A = q.cp[k];
                Vec3 XA{P.X[3 * A], P.X[3 * A + 1], P.X[3 * A + 2]};
                Vec3 uA{ufull[A], ufull[ncp + A], ufull[2 * ncp + A]};
                X11 = X11 + q.N11[k] * XA; X22 = X22 + q.N22[k] * XA; X12 = X12 + q.N12[k] * XA;
                d1 = d1 + q.N1[k] * uA; d2 = d2 + q.N2[k] * uA;
                d11 = d11 + q.N11[k] * uA; d22 = d22 + q.N22[k] * uA; d12 = d12 + q.N12[k] * uA;
            }
            Vec3 a1 = A1 + d1, a2 = A2 + d2, x11 = X11 + d11, x22 = X22 + d22, x12 = X12 + d12;
            Vec3 At = cross(A1, A2);
            double J0 = std::sqrt(dot(At, At));
            Vec3 A3 = (1.0 / J0) * At;
            Vec3 at = cross(a1, a2);
            double l = std::sqrt(dot(at, at));
            Vec3 a3 = (1.0 / l) * at;
            double Am[3] = {dot(A1, A1), dot(A2, A2), dot(A1, A2)};
            double am[3] = {dot(a1, a1), dot(a2, a2), dot(a1, a2)};
            double Bc[3] = {dot(X11, A3), dot(X22, A3), dot(X12, A3)};
            double bc[3] = {dot(x11, a3), dot(x22, a3), dot(x12, a3)};
            // membrane strain from the displacement gradient d_a = a_a - A_a (the same value as
            // 1/2 (a_ab - A_ab) without the cancellation of two nearly equal metrics)
            double eps[3] = {dot(A1, d1) + 0.5 * dot(d1, d1), dot(A2, d2) + 0.5 * dot(d2, d2),
                             dot(A1, d2) + dot(d1, A2) + dot(d1, d2)};
            (void)am;
            double kap[3] = {Bc[0] - bc[0], Bc[1] - bc[1], 2.0 * (Bc[2] - bc[2])};
            double C[3][3];
            material(P, Am[0], Am[2], Am[1], C);
            double tm = P.t, tb = P.t * P.t * P.t / 12.0;
            double nv[3], mv[3];
            for (int r = 0; r < 3; ++r) {
                nv[r] = tm * (C[r][0] * eps[0] + C[r][1] * eps[1] + C[r][2] * eps[2]);
                mv[r] = tb * (C[r][0] * kap[0] + C[r][1] * kap[1] + C[r][2] * kap[2]);
            }
            double dV = q.dA;
            // first variations, dof by dof
            double dE[MAXD][3], dK[MAXD][3];
            Vec3 dat[MAXD], da3[MAXD];
            double dl[MAXD];
            for (int k = 0; k < nb; ++k)
                for (int i = 0; i < 3; ++i) {
                    int r = 3 * k + i;
                    Vec3 ei = unit(i);
                    dE[r][0] = q.N1[k] * comp(a1, i);
                    dE[r][1] = q.N2[k] * comp(a2, i);
                    dE[r][2] = q.N1[k] * comp(a2, i) + q.N2[k] * comp(a1, i);
                    dat[r] = q.N1[k] * cross(ei, a2) + q.N2[k] * cross(a1, ei);
                    dl[r] = dot(a3, dat[r]);
                    da3[r] = (1.0 / l) * (dat[r] - dl[r] * a3);
                    double db11 = q.N11[k] * comp(a3, i) + dot(x11, da3[r]);
                    double db22 = q.N22[k] * comp(a3, i) + dot(x22, da3[r]);
                    double db12 = q.N12[k] * comp(a3, i) + dot(x12, da3[r]);
                    dK[r][0] = -db11; dK[r][1] = -db22; dK[r][2] = -2.0 * db12;
                    Fe[r] += (nv[0] * dE[r][0] + nv[1] * dE[r][1] + nv[2] * dE[r][2] +
                              mv[0] * dK[r][0] + mv[1] * dK[r][1] + mv[2] * dK[r][2]) * dV;
                }
            if (!wantK) continue;
            double CdE[MAXD][3], CdK[MAXD][3];
            for (int r = 0; r < d; ++r)
                for (int a = 0; a < 3; ++a) {
                    CdE[r][a] = tm * (C[a][0] * dE[r][0] + C[a][1] * dE[r][1] + C[a][2] * dE[r][2]);
                    CdK[r][a] = tb * (C[a][0] * dK[r][0] + C[a][1] * dK[r][1] + C[a][2] * dK[r][2]);
                }
            for (int kr = 0; kr < nb; ++kr)
                for (int i = 0; i < 3; ++i) {
                    int r = 3 * kr + i;
                    for (int ks = 0; ks < nb; ++ks)
                        for (int j = 0; j < 3; ++j) {
                            int s = 3 * ks + j;
                            double v = CdE[r][0] * dE[s][0] + CdE[r][1] * dE[s][1] + CdE[r][2] * dE[s][2] +
                                       CdK[r][0] * dK[s][0] + CdK[r][1] * dK[s][1] + CdK[r][2] * dK[s][2];
                            // membrane second variation
                            if (i == j)
                                v += nv[0] * q.N1[kr] * q.N1[ks] + nv[1] * q.N2[kr] * q.N2[ks] +
                                     nv[2] * (q.N1[kr] * q.N2[ks] + q.N2[kr] * q.N1[ks]);
                            // bending second variation
                            Vec3 ddat = q.N1[kr] * q.N2[ks] * cross(unit(i), unit(j)) +
                                        q.N1[ks] * q.N2[kr] * cross(unit(j), unit(i));
                            double ddl = dot(da3[r], dat[s]) + dot(a3, ddat);
                            Vec3 dda3 = (1.0 / l) * (ddat - dl[s] * da3[r] - dl[r] * da3[s] - ddl * a3);
                            double ddb11 = q.N11[kr] * comp(da3[s], i) + q.N11[ks] * comp(da3[r], j) + dot(x11, dda3);
                            double ddb22 = q.N22[kr] * comp(da3[s], i) + q.N22[ks] * comp(da3[r], j) + dot(x22, dda3);
                            double ddb12 = q.N12[kr] * comp(da3[s], i) + q.N12[ks] * comp(da3[r], j) + dot(x12, dda3);
                            v -= mv[0] * ddb11 + mv[1] * ddb22 + 2.0 * mv[2] * ddb12;
                            Ke[r * d + s] += v * dV;
                        }
                }
        }
}

// Full-space CSR pattern: row (c, A=(i,j)), columns (c', B=(i',j')) with |i-i'|<=p, |j-j'|<=p,
// sorted by c' then j' then i'.
struct Pattern {
    int n1, n2, p, ncp;
    std::vector<int64_t> rowptr;
    int ilo(int i) const { return std::max(0, i - p); }
    int ihi(int i) const { return std::min(n1 - 1, i + p); }
    int jlo(int j) const { return std::max(0, j - p); }
    int jhi(int j) const { return std::min(n2 - 1, j + p); }
    void build() {
        ncp = n1 * n2;
        rowptr.assign(3 * (size_t)ncp + 1, 0);
        for (int c = 0; c < 3; ++c)
            for (int A = 0; A < ncp; ++A) {
                int i = A % n1, j = A / n1;
                int cnt = (ihi(i) - ilo(i) + 1) * (jhi(j) - jlo(j) + 1) * 3;
                rowptr[(size_t)c * ncp + A + 1] = cnt;
            }
        for (size_t r = 0; r < 3 * (size_t)ncp; ++r) rowptr[r + 1] += rowptr[r];
    }
    int64_t pos(int c, int A, int c2, int B) const {
        int i = A % n1, j = A / n1, i2 = B % n1, j2 = B / n1;
        int ci = ihi(i) - ilo(i) + 1, cj = jhi(j) - jlo(j) + 1;
        return rowptr[(size_t)c * ncp + A] + (int64_t)c2 * ci * cj + (int64_t)(j2 - jlo(j)) * ci + (i2 - ilo(i));
    }
    void cols(int32_t* out) const {
        for (int c = 0; c < 3; ++c)
            for (int A = 0; A < ncp; ++A) {
                int i = A % n1, j = A / n1;
                int64_t k = rowptr[(size_t)c * ncp + A];
                for (int c2 = 0; c2 < 3; ++c2)
                    for (int j2 = jlo(j); j2 <= jhi(j); ++j2)
                        for (int i2 = ilo(i); i2 <= ihi(i); ++i2) out[k++] = c2 * ncp + j2 * n1 + i2;
            }
    }
};

Patch make_patch(int p, int n1, int n2, const double* U1, const double* U2, const double* X,
                 double E, double nu, double t, double rho, int nq) {
    Patch P;
    P.p = p; P.n1 = n1; P.n2 = n2; P.U1 = U1; P.U2 = U2; P.X = X;
    P.E = E; P.nu = nu; P.t = t; P.rho = rho; P.nq = nq > 0 ? nq : p + 1;
    return P;
}

// colour of element (s1, s2): elements of one colour share no control point
int colour(const Patch& P, const Elem& e) { return (e.s1 % (P.p + 1)) * (P.p + 1) + (e.s2 % (P.p + 1)); }

}  // namespace

extern "C" {

// Number of nonzeros of the full-space (3*n1*n2 square) CSR pattern.
int64_t klo_full_nnz(int p, int n1, int n2) {
    Pattern pt{n1, n2, p, 0, {}};
    pt.build();
    return pt.rowptr.back();
}

// Full-space CSR pattern (rowptr: 3*n1*n2+1, cols: nnz).
void klo_full_pattern(int p, int n1, int n2, int64_t* rowptr, int32_t* cols) {
    Pattern pt{n1, n2, p, 0, {}};
    pt.build();
    std::memcpy(rowptr, pt.rowptr.data(), pt.rowptr.size() * sizeof(int64_t));
    pt.cols(cols);
}

// Tangent K(u) (values in the full pattern, may be null) and internal force Fint(u)
// (full layout, may be null) at full displacement u (component-blocked).
int klo_assemble(int p, int n1, int n2, const double* U1, const double* U2, const double* X,
                 double E, double nu, double t, int nq, const double* ufull, double* Kvals, double* fint,
                 int nthreads, const double* weights) {
    if (p < 1 || p > MAXP) return -1;
    Patch P = make_patch(p, n1, n2, U1, U2, X, E, nu, t, 0.0, nq);
    P.W = weights;
    Pattern pt{n1, n2, p, 0, {}};
    pt.build();
    int ncp = n1 * n2;
    if (Kvals) std::memset(Kvals, 0, sizeof(double) * pt.rowptr.back());
    if (fint) std::memset(fint, 0, sizeof(double) * 3 * ncp);
    std::vector<Elem> els = elements(P);
    int ncol = (p + 1) * (p + 1);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    for (int col = 0; col < ncol; ++col) {
#pragma omp parallel
        {
            std::vector<double> Ke, Fe;
#pragma omp for schedule(dynamic, 4)
            for (long ie = 0; ie < (long)els.size(); ++ie) {
                const Elem& e = els[ie];
                if (colour(P, e) != col) continue;
                int nb;
                element_kl(P, e, ufull, ncp, Kvals != nullptr, Ke, Fe, nb);
                int nb1 = p + 1;
                int cps[MAXB * MAXB];
                for (int b = 0; b < nb1; ++b)
                    for (int a = 0; a < nb1; ++a) cps[b * nb1 + a] = (e.s2 - p + b) * n1 + (e.s1 - p + a);
                int d = 3 * nb;
                for (int kr = 0; kr < nb; ++kr)
                    for (int i = 0; i < 3; ++i) {
                        int r = 3 * kr + i;
                        if (fint) fint[(size_t)i * ncp + cps[kr]] += Fe[r];
                        if (!Kvals) continue;
                        for (int ks = 0; ks < nb; ++ks)
                            for (int j = 0; j < 3; ++j)
                                Kvals[pt.pos(i, cps[kr], j, cps[ks])] += Ke[r * d + 3 * ks + j];
                    }
            }
        }
    }
    return 0;
}

// Consistent mass matrix M = int rho t N_A N_B dA (identity in the components) in the full pattern.
int klo_mass(int p, int n1, int n2, const double* U1, const double* U2, const double* X, double rho, double t,
             int nq, double* Mvals, const double* weights) {
    Patch P = make_patch(p, n1, n2, U1, U2, X, 1.0, 0.0, t, rho, nq);
    P.W = weights;
    Pattern pt{n1, n2, p, 0, {}};
    pt.build();
    std::memset(Mvals, 0, sizeof(double) * pt.rowptr.back());
    double gx[16], gw[16];
    gauss_legendre(P.nq, gx, gw);
    for (const Elem& e : elements(P)) {
        double jac = 0.25 * (e.u1 - e.u0) * (e.v1 - e.v0);
        for (int q2 = 0; q2 < P.nq; ++q2)
            for (int q1 = 0; q1 < P.nq; ++q1) {
                QP q;
                Vec3 A1, A2;
                double xi1 = 0.5 * (e.u0 + e.u1) + 0.5 * (e.u1 - e.u0) * gx[q1];
                double xi2 = 0.5 * (e.v0 + e.v1) + 0.5 * (e.v1 - e.v0) * gx[q2];
                eval_qp(P, e, xi1, xi2, gw[q1] * gw[q2] * jac, q, A1, A2);
                for (int a = 0; a < q.nb; ++a)
                    for (int b = 0; b < q.nb; ++b) {
                        double v = rho * t * q.N[a] * q.N[b] * q.dA;
                        for (int c = 0; c < 3; ++c) Mvals[pt.pos(c, q.cp[a], c, q.cp[b])] += v;
                    }
            }
    }
    return 0;
}

// External load vector (full layout): dead surface load qsurf (per reference area, 3 comps),
// point loads (npl x [xi1, xi2, Px, Py, Pz]) and edge line loads (ned x [side, qx, qy, qz],
// side 0: xi1=0, 1: xi1=1, 2: xi2=0, 3: xi2=1; per unit reference length).
int klo_force(int p, int n1, int n2, const double* U1, const double* U2, const double* X, int nq,
              const double* qsurf, int npl, const double* pl, int ned, const double* ed, double* F,
              const double* weights) {
    Patch P = make_patch(p, n1, n2, U1, U2, X, 1.0, 0.0, 1.0, 0.0, nq);
    P.W = weights;
    int ncp = n1 * n2;
    std::memset(F, 0, sizeof(double) * 3 * ncp);
    double gx[16], gw[16];
    gauss_legendre(P.nq, gx, gw);
    if (qsurf && (qsurf[0] != 0 || qsurf[1] != 0 || qsurf[2] != 0)) {
        for (const Elem& e : elements(P)) {
            double jac = 0.25 * (e.u1 - e.u0) * (e.v1 - e.v0);
            for (int q2 = 0; q2 < P.nq; ++q2)
                for (int q1 = 0; q1 < P.nq; ++q1) {
                    QP q;
                    Vec3 A1, A2;
                    double xi1 = 0.5 * (e.u0 + e.u1) + 0.5 * (e.u1 - e.u0) * gx[q1];
                    double xi2 = 0.5 * (e.v0 + e.v1) + 0.5 * (e.v1 - e.v0) * gx[q2];
                    eval_qp(P, e, xi1, xi2, gw[q1] * gw[q2] * jac, q, A1, A2);
                    for (int a = 0; a < q.nb; ++a)
                        for (int c = 0; c < 3; ++c) F[(size_t)c * ncp + q.cp[a]] += q.N[a] * qsurf[c] * q.dA;
                }
        }
    }
    for (int k = 0; k < npl; ++k) {
        const double* L = pl + 5 * k;
        int s1, s2;
        double b1[3][MAXB], b2[3][MAXB];
        basis_ders(n1, p, U1, L[0], s1, b1);
        basis_ders(n2, p, U2, L[1], s2, b2);
        double Wp = 1.0;
        if (weights) {
            Wp = 0.0;
            for (int b = 0; b <= p; ++b)
                for (int a = 0; a <= p; ++a) Wp += weights[(s2 - p + b) * n1 + (s1 - p + a)] * b1[0][a] * b2[0][b];
        }
        for (int b = 0; b <= p; ++b)
            for (int a = 0; a <= p; ++a) {
                int A = (s2 - p + b) * n1 + (s1 - p + a);
                const double R = (weights ? weights[A] / Wp : 1.0) * b1[0][a] * b2[0][b];
                for (int c = 0; c < 3; ++c) F[(size_t)c * ncp + A] += R * L[2 + c];
            }
    }
    for (int k = 0; k < ned; ++k) {
        const double* L = ed + 4 * k;
        int side = (int)L[0];
        bool along1 = (side >= 2);              // edge runs along parameter 1
        const double* Ue = along1 ? U1 : U2;
        int ne = along1 ? n1 : n2;
        double fixed = (side == 0 || side == 2) ? 0.0 : 1.0;
        for (int s = p; s < ne; ++s) {
            if (!(Ue[s + 1] > Ue[s])) continue;
            double jac = 0.5 * (Ue[s + 1] - Ue[s]);
            for (int qq = 0; qq < P.nq; ++qq) {
                double t = 0.5 * (Ue[s] + Ue[s + 1]) + jac * gx[qq];
                double xi1 = along1 ? t : fixed, xi2 = along1 ? fixed : t;
                int s1, s2;
                double b1[3][MAXB], b2[3][MAXB];
                basis_ders(n1, p, U1, xi1, s1, b1);
                basis_ders(n2, p, U2, xi2, s2, b2);
                // values and edge-direction derivatives of the (rational) basis
                double Rv[MAXB * MAXB], Rt[MAXB * MAXB];
                double We = 0.0, Wt = 0.0;
                for (int b = 0; b <= p; ++b)
                    for (int a = 0; a <= p; ++a) {
                        const int k = b * (p + 1) + a, A = (s2 - p + b) * n1 + (s1 - p + a);
                        Rv[k] = b1[0][a] * b2[0][b];
                        Rt[k] = along1 ? b1[1][a] * b2[0][b] : b1[0][a] * b2[1][b];
                        const double w = weights ? weights[A] : 1.0;
                        We += w * Rv[k];
                        Wt += w * Rt[k];
                    }
                if (weights)
                    for (int b = 0; b <= p; ++b)
                        for (int a = 0; a <= p; ++a) {
                            const int k = b * (p + 1) + a, A = (s2 - p + b) * n1 + (s1 - p + a);
                            const double c = weights[A] / We;
                            Rt[k] = c * (Rt[k] - Rv[k] * Wt / We);
                            Rv[k] = c * Rv[k];
                        }
                Vec3 T{0, 0, 0};
                for (int b = 0; b <= p; ++b)
                    for (int a = 0; a <= p; ++a) {
                        int A = (s2 - p + b) * n1 + (s1 - p + a);
                        T = T + Rt[b * (p + 1) + a] * Vec3{X[3 * A], X[3 * A + 1], X[3 * A + 2]};
                    }
                double ds = std::sqrt(dot(T, T)) * jac * gw[qq];
                for (int b = 0; b <= p; ++b)
                    for (int a = 0; a <= p; ++a) {
                        int A = (s2 - p + b) * n1 + (s1 - p + a);
                        double Nv = Rv[b * (p + 1) + a];
                        for (int c = 0; c < 3; ++c) F[(size_t)c * ncp + A] += Nv * L[1 + c] * ds;
                    }
            }
        }
    }
    return 0;
}

// B-spline values/derivatives (testing hook): out[3*(p+1)] = N, N', N'' of functions span-p..span.
int klo_basis(int p, int ncp, const double* U, double u, double* out) {
    int span;
    double b[3][MAXB];
    basis_ders(ncp, p, U, u, span, b);
    for (int d = 0; d < 3; ++d)
        for (int a = 0; a <= p; ++a) out[d * (p + 1) + a] = b[d][a];
    return span;
}

}  // extern "C"
