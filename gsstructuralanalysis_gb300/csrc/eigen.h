// eigen.h -- shift-invert Lanczos for the buckling and modal pencils (Spectra stand-in).
#pragma once

#include "problem.h"
#include "solvers.h"

namespace klsa {

// gsBucklingSolver (gsEigenSolvers/gsBucklingSolver.h:127-149) + Spectra Buckling mode
// (gsEigenProblemBase.hpp:152-215): u_L = K_L^-1 (s F), B = K(u_L) - K_L, K_L v = lambda B v.
int buckling_gpu(Problem& P, const Options& opt, int nev, double shift, double scaling, double* values,
                 double* vectors);
// gsModalSolver (gsEigenSolvers/gsModalSolver.h:46-51) + Spectra ShiftInvert mode: K v = lambda M v.
int modal_gpu(Problem& P, const Options& opt, int nev, double shift, double* values, double* vectors);

// y = A x with an explicit FP64 value array over the problem's CSR pattern
void spmv_vals(const Problem& P, const double* vals, const double* x, double* y);

}  // namespace klsa
