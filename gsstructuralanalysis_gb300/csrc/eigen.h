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

// Standard symmetric problem A v = lambda v in shift-invert mode, the stability indicator of
// gsALMBase::_computeStability (gsALMSolvers/gsALMBase.hpp:570-598): Spectra SymShiftSolver with
// ncv = ncv_fac * nev, selection LargestAlge of nu = 1/(lambda - shift), values returned ascending
// (SmallestAlge).  valsA: FP64 values on the problem's CSR pattern.  Uses the problem's
// factorisation workspace (the caller's factorisation is overwritten).
int standard_eigs_gpu(Problem& P, const double* valsA, int nev, int ncv_fac, double shift, double tol, double* values);

// gsEigenProblemBase::computePower of the modal (kind 0) or buckling (kind 1) pencil: the
// eigenpair of smallest |lambda| by power iteration on A^-1 B (gsEigenProblemBase.hpp:218-258).
int power_gpu(Problem& P, const Options& opt, int kind, double scaling, double* value, double* vector);

// gsEigenProblemBase::compute of the modal (kind 0) or buckling (kind 1) pencil: every eigenpair
// of the dense pencil (gsEigenProblemBase.hpp:21-50).  values: ndof, vectors: ndof x ndof.
int dense_gpu(Problem& P, const Options& opt, int kind, double scaling, double* values, double* vectors);

// y = A x with an explicit FP64 value array over the problem's CSR pattern
void spmv_vals(const Problem& P, const double* vals, const double* x, double* y);

}  // namespace klsa
