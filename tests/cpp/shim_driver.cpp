// C++ driver of the header-only layer (include/klshell_gb300.hpp): builds a 2x2-element simply
// supported plate (degree 2, boundary control points fixed), and either solves it with
// gsStaticNewton's mirror and prints the free-dof solution (a device is present) or reports the
// library's CUDA error through klsa::Error (no device).  Checks ABI error handling on every path.
#include <cstdio>
#include <vector>

#include "klshell_gb300.hpp"

int main() {
    const int p = 2, n = 4;
    std::vector<double> knots = {0, 0, 0, 0.5, 1, 1, 1};
    const double g[4] = {0.0, 0.25, 0.75, 1.0};   // Greville abscissae: a flat, affinely mapped net
    std::vector<double> ctrl;
    std::vector<uint8_t> fixed(3 * n * n, 0);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            ctrl.insert(ctrl.end(), {g[i], g[j], 0.0});
            const bool bnd = i == 0 || j == 0 || i == n - 1 || j == n - 1;
            for (int c = 0; c < 3; ++c) fixed[c * n * n + j * n + i] = bnd ? 1 : 0;
        }
    const double q[3] = {0.0, 0.0, 1.0};
    klsa_patch_desc d = {};
    d.p = p; d.n1 = n; d.n2 = n; d.nq = 0;
    d.knots1 = knots.data(); d.knots2 = knots.data(); d.ctrl = ctrl.data();
    d.E = 1e7; d.nu = 0.3; d.thickness = 0.01; d.density = 1.0;
    d.fixed = fixed.data(); d.surface_load = q;

    // argument errors surface as klsa::Error with the ABI code
    try {
        klsa::check(klsa_alm_create(nullptr, "Crisfield", nullptr, nullptr));
        std::printf("missing-error\n");
        return 1;
    } catch (const klsa::Error& e) {
        if (e.code != KLSA_INVALID_ARGUMENT) return 1;
    }
    klsa::Options o;
    o.setString("Solver", "SimplicialLDLT").setReal("tol", 1e-10).setInt("maxIt", 20);
    try {
        klsa::Problem P(d);
        klsa::StaticNewton N(P, o);
        const int st = N.solve();
        const std::vector<double> U = N.solution();
        double wmax = 0.0;
        for (double v : U) wmax = v > wmax ? v : wmax;
        std::printf("ok status=%d ndof=%lld wmax=%.6e\n", st, (long long)P.numDofs(), wmax);
        std::printf("U");
        for (double v : U) std::printf(" %.17e", v);
        std::printf("\n");
        return st == 0 ? 0 : 1;
    } catch (const klsa::Error& e) {
        std::printf("no-device code=%d\n", e.code);
        return e.code == KLSA_CUDA_ERROR ? 0 : 1;
    }
}
