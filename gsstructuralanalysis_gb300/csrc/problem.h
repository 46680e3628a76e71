// problem.h -- one Kirchhoff-Love shell patch resident on the device.
//
// HBM layout (per problem)
//   tab1/tab2   1-D B-spline values and 1st/2nd derivatives at the Gauss points of every
//               element column/row: [m][nq][3][p+1] (FP64 and FP32 copies)
//   qpgeo       per Gauss point (QGEO = 25 values): A1, A2, X,11, X,22, X,12 (reference, 15),
//               the SVK material matrix in the contravariant reference metric (6), the area
//               weight (1) and the reference curvature coefficients X,11.A3, X,22.A3, X,12.A3
//               (3), FP64
//   u_full      displacement in the component-blocked full layout, FP64
//   elemK/elemR element tangents (d x d) and internal forces (d) of the last assembly
//   CSR         rows = free dofs in internal (nested-dissection) order, int32 cols,
//               FP32 and/or FP64 values
// Internal order = postorder of the nested-dissection tree; the public (reference) order is
// component-blocked free dofs.  Both permutations are kept on the device.
#pragma once

#include <cuda_runtime.h>
#include <memory>
#include <vector>

#include "common.cuh"

namespace klsa {
constexpr int QGEO = 25;   // values per Gauss point in qpgeo
}
#include "multifrontal.h"
#include "nd_symbolic.h"

struct klsa_patch_desc;

namespace klsa {

struct Problem {
    // description
    int p = 0, n1 = 0, n2 = 0, nq = 0, ncp = 0, m1 = 0, m2 = 0, nel = 0, nqp = 0;
    double E = 0, nu = 0, t = 0, rho = 0;
    std::vector<double> U1, U2, X;
    std::vector<uint8_t> fixed;
    int nfree = 0;
    int64_t nnz = 0;

    NDTree tree;
    std::vector<int> rowptr, cols;     // internal order
    std::vector<int> pub2int, int2pub;
    std::vector<double> F_int_order;   // external load (internal order)

    cudaStream_t stream = nullptr;
    DevBuf<double> d_tab1, d_tab2, d_qpgeo;
    DevBuf<float> d_tab1f, d_tab2f;
    DevBuf<float2> d_tab1s, d_tab2s;       // basis tables as FP32 hi/lo pairs (double-float residual)
    bool fint_fp64 = false;                // internal force: plain FP64 kernel instead of double-float sums
    DevBuf<int> d_int2full, d_full2int, d_pub2int, d_int2pub;
    DevBuf<int> d_rowptr, d_cols;
    DevBuf<double> d_F;                // external load, internal order
    DevBuf<double> d_ufull;
    DevBuf<float> d_elemKf;
    DevBuf<double> d_elemKd, d_elemR;
    DevBuf<float> d_vals32;
    DevBuf<double> d_vals64, d_fint;
    DevBuf<double> d_tmp_pub;          // host-boundary staging (public order)
    DevBuf<double> d_tmp_int;

    std::unique_ptr<Multifrontal> mf;
    std::unique_ptr<Multifrontal64> mf64;

    explicit Problem(const klsa_patch_desc& d);
    ~Problem();

    // --- device operations (internal order, device pointers) ---------------------------
    void set_displacement(const double* d_x);           // u_full <- x (free dofs)
    void set_displacement_sum(const double* a, const double* b, double* x);   // x = a + b; u_full <- x
    void tangent_f32();                                 // d_vals32 = K(u) (FP32 element integration)
    void tangent_f64();                                 // d_vals64 = K(u) (FP64)
    // Fint(u) + (alpha - *alpha_sub) y (y and alpha_sub may be null), internal order, FP64
    void internal_force(double* d_out, double alpha = 0.0, const double* y = nullptr, const double* alpha_sub = nullptr);
    void internal_force_elements(double* elemR);        // element forces of u into elemR (nel*d), no allocation
    void mass_f64();                                    // d_vals64 = M
    Multifrontal& solver();                             // lazily built (FP32 fronts)
    Multifrontal64& solver64();                         // lazily built (FP64 fronts)

    // public <-> internal permutations of nv vectors (device)
    void pub_to_int(const double* d_pub, double* d_int, int nv = 1);
    void int_to_pub(const double* d_int, double* d_pub, int nv = 1);
    // host helpers
    void upload_pub(const double* h_pub, double* d_int, int nv = 1);
    void download_pub(const double* d_int, double* h_pub, int nv = 1);
    void csr_to_host_pub(bool f64, int64_t* rowptr_out, int32_t* cols_out, double* vals_out);

    double flops_tangent() const;   // algorithmic flops of one tangent assembly
};

// vector kernels (device, FP64 unless noted)
namespace vec {
void to_f32(const double* x, float* y, int64_t n, cudaStream_t s);
void to_f64(const float* x, double* y, int64_t n, cudaStream_t s);
void axpby(double a, const double* x, double b, double* y, int64_t n, cudaStream_t s);   // y = a x + b y
void lincomb(double a, const double* x, double b, const double* y, double* z, int64_t n, cudaStream_t s);  // z = a x + b y
// z = a x + b y, and also z2 = z (z2 given) and acc += z (acc given)
void lincomb_ext(double a, const double* x, double b, const double* y, double* z, double* z2, double* acc, int64_t n,
                 cudaStream_t s);
void step_finish(double* u, const double* d, double* uprev, double* dold, int64_t n, cudaStream_t s);  // uprev = u; u += d; dold = d
void zero4(double* a, double* b, double* c, double* d, int64_t n, cudaStream_t s);   // null pointers skipped
// dots[i] = <x_i, y_i> for up to 8 pairs, FP64, result copied to host (synchronises)
void multidot(int npairs, const double* const* xs, const double* const* ys, int64_t n, double* host_out,
              cudaStream_t s);
}  // namespace vec

// CSR SpMV: y = A x (FP32 or FP64 values, FP64 vectors)
void spmv(const Problem& P, bool f64, const double* x, double* y);

}  // namespace klsa
