/* klshell_gb300.h -- C-ABI of the GB300 (sm_103a) Kirchhoff-Love shell hot path.
 *
 * The reference module (gsStructuralAnalysis) has no FFI: its boundary is the set of C++
 * callback types in gsStructuralAnalysisTools/gsStructuralAnalysisTypes.h:58-93
 * (Jacobian_t, dJacobian_t, Residual_t, ALResidual_t, Mass_t, Force_t), the sparse-solver
 * name resolved by gsSparseSolver<T>::get (gsStaticSolvers/gsStaticBase.h:85,
 * gsALMSolvers/gsALMBase.hpp:73) and the solver classes' step/solve calls.  Each entry
 * point below names the reference interface it replaces.  Plain pointers and sizes only;
 * host buffers are caller-owned; every call returns a status (0..5 = gsStatus, negative =
 * ABI error) and never throws.
 *
 * Vector layout of every host vector: free dofs in the reference's order (component-blocked
 * x,y,z, Dirichlet dofs removed), i.e. what gsThinShellAssembler's Residual/Jacobian
 * callbacks exchange with the solvers.
 */
#ifndef KLSHELL_GB300_H
#define KLSHELL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (gsStatus, gsStructuralAnalysisTypes.h:22-30) ---------------------- */
#define KLSA_SUCCESS 0
#define KLSA_NOT_CONVERGED 1
#define KLSA_ASSEMBLY_ERROR 2
#define KLSA_SOLVER_ERROR 3
#define KLSA_NOT_STARTED 4
#define KLSA_OTHER_ERROR 5
#define KLSA_INVALID_ARGUMENT (-1)
#define KLSA_CUDA_ERROR (-2)
#define KLSA_UNSUPPORTED (-3)

/* ---- problem description ------------------------------------------------------------- */
/* One tensor-product B-spline patch (open knot vectors, simple interior knots), SVK
 * material, homogeneous Dirichlet mask, dead loads.  Control point A = j*n1 + i. */
typedef struct klsa_patch_desc {
    int32_t p;                   /* degree in both directions, 1..4 */
    int32_t n1, n2;              /* control points per direction */
    int32_t nq;                  /* Gauss points per direction per element, 0 -> p+1 */
    const double* knots1;        /* n1+p+1 */
    const double* knots2;        /* n2+p+1 */
    const double* ctrl;          /* n1*n2*3 reference control points, (A*3 + c) */
    double E, nu, thickness, density;
    const uint8_t* fixed;        /* 3*n1*n2 component-blocked mask, 1 = Dirichlet (u = 0) */
    const double* surface_load;  /* 3 comps per unit reference area, or NULL */
    int32_t n_point_loads;       /* rows of [xi1, xi2, Px, Py, Pz] */
    const double* point_loads;
    int32_t n_edge_loads;        /* rows of [side(0:xi1=0,1:xi1=1,2:xi2=0,3:xi2=1), qx, qy, qz] */
    const double* edge_loads;
} klsa_patch_desc;

typedef struct klsa_problem klsa_problem;
typedef struct klsa_options klsa_options;
typedef struct klsa_solver klsa_solver;
typedef struct klsa_static klsa_static;
typedef struct klsa_alm klsa_alm;

/* Last error message of the calling thread (static storage). */
const char* klsa_last_error(void);
/* Number of CUDA kernels this library launched since load (graph replays count their nodes). */
uint64_t klsa_launch_count(void);

/* Builds device geometry tables, the dof maps, the CSR pattern and the nested-dissection
 * analysis.  Replaces constructing gsThinShellAssembler + assemble() (call sites
 * tutorials/nonlinear_shell_static.cpp:106-139). */
int klsa_problem_create(const klsa_patch_desc* desc, klsa_problem** out);
int klsa_problem_destroy(klsa_problem* prob);
int64_t klsa_problem_ndof(const klsa_problem* prob);   /* free dofs */
int64_t klsa_problem_nnz(const klsa_problem* prob);    /* CSR nonzeros of K over free dofs */

/* Force_t (gsStructuralAnalysisTypes.h:61): external load vector F. */
int klsa_force(klsa_problem* prob, double* F);
/* Residual_t (Types.h:66): R = Fext - Fint(x), assembled in FP64 on the device. */
int klsa_residual(klsa_problem* prob, const double* x, double* R);
/* ALResidual_t (Types.h:68): R = Fint(x) - lambda*F (tutorials/nonlinear_shell_arcLength.cpp:135-142). */
int klsa_al_residual(klsa_problem* prob, const double* x, double lambda, double* R);
/* Jacobian_t (Types.h:85): K(x) as CSR over free dofs (reference order, rows sorted).
 * precision 0: FP32 element integration, 1: FP64.  rowptr has ndof+1 entries. */
int klsa_jacobian_csr(klsa_problem* prob, const double* x, int precision, int64_t* rowptr, int32_t* cols,
                      double* vals);
/* dJacobian_t (Types.h:91-92): the Jacobian with the solution update as an extra argument, as
 * gsALMBase::_computeJacobian (gsALMBase.hpp:214-223) and gsStaticNewton::_computeJacobian
 * (gsStaticNewton.hpp:205-212) call it.  Same output as klsa_jacobian_csr at x: for the SVK
 * material the tangent does not depend on dx, exactly as the reference wraps a Jacobian_t into
 * its dJacobian_t (gsALMBase.h:57-60, gsStaticNewton.h:79-82).  dx: ndof values (must be given). */
int klsa_djacobian_csr(klsa_problem* prob, const double* x, const double* dx, int precision, int64_t* rowptr,
                       int32_t* cols, double* vals);
/* Mass_t (Types.h:71): consistent mass matrix int rho t N_A N_B dA, same CSR pattern. */
int klsa_mass_csr(klsa_problem* prob, int64_t* rowptr, int32_t* cols, double* vals);

/* ALResidual_t without device allocation -- no counterpart in the reference.  For callers that
 * must not allocate device memory at the point where they need a residual: a host framework
 * that owns the whole device memory pool and forbids allocations outside it, or a
 * memory-budgeted service whose device footprint is fixed when it starts.  The regular
 * klsa_al_residual grows its element-force and staging buffers with cudaMalloc on first use;
 * this one does not.  x and R are caller-owned DEVICE vectors in the public free-dof order.
 *   - Scratch: a fixed file-scope device array of 2^20 doubles (8 MiB on every GPU that loads
 *     the library, held until exit).  Problems needing more than 2^20 element-force entries
 *     (elements x 3(p+1)^2) are rejected with KLSA_INVALID_ARGUMENT.
 *   - Every call shares that array and it keeps the last call's contents; calls that overlap on
 *     the GPU (two host threads, or two problems) race on it: serialise them.
 *   - The call also overwrites the problem's own displacement state (the full-layout vector
 *     that klsa_residual / klsa_al_residual and the solvers of this problem write), so it must
 *     not overlap any other call on the same problem.
 *   - The kernels run on the problem's own stream, which does not wait for other streams: all
 *     pending writes to x must be complete before the call (synchronise the stream that wrote
 *     it).  The call synchronises the problem's stream before it returns, so R is ready then.
 *   - The first call on a device resolves the array's device address once
 *     (cudaGetSymbolAddress, with that device current). */
int klsa_al_residual_noalloc(klsa_problem* prob, const double* d_x, double lambda, double* d_R);

/* ---- options (gsOptionList keys and defaults of the mirrored classes) ------------------ */
klsa_options* klsa_options_create(void);
void klsa_options_destroy(klsa_options* opt);
int klsa_options_set_real(klsa_options* opt, const char* key, double value);
int klsa_options_set_int(klsa_options* opt, const char* key, int64_t value);
int klsa_options_set_string(klsa_options* opt, const char* key, const char* value);

/* ---- named sparse solver (gsSparseSolver<T>::get(name), gsStaticBase.h:85) --------------
 * "SimplicialLDLT" / "GPUMultifrontalLDLT": nested-dissection multifrontal LDL^T, FP32
 * fronts, optional FP64 iterative refinement ("Refinement" steps, tolerance "RefineTol").
 * "CGDiagonal": Jacobi-preconditioned CG on the CSR matrix (Eigen's ConjugateGradient with the
 * DiagonalPreconditioner); "GPUPCG" / "BlockJacobiCG": CG with the nodal 3x3 block-Jacobi
 * preconditioner.  Options "CGMaxIterations" (default 2 ndof) and "CGTolerance". */
int klsa_solver_create(klsa_problem* prob, const char* name, const klsa_options* opt, klsa_solver** out);
int klsa_solver_destroy(klsa_solver* s);
/* compute(K(x)) of the named solver: assemble the tangent at x on the device and factorise. */
int klsa_solver_compute_jacobian(klsa_solver* s, const double* x);
/* compute(K_L) */
int klsa_solver_compute_linear(klsa_solver* s);
/* solve(b) for nrhs right-hand sides stored one after the other (ndof each). */
int klsa_solver_solve(klsa_solver* s, const double* b, double* x, int nrhs);
/* Iterations of the last solve: CG iterations (the PCG solvers) or refinement sweeps (LDL^T). */
int klsa_solver_iterations(klsa_solver* s);
/* LDL^T pivots: minimum of D and number of negative entries (determinant stability
 * indicator, gsStaticBase.h:162-179). */
int klsa_solver_stability(klsa_solver* s, double* min_d, int64_t* negatives);

/* ---- gsStaticNewton (gsStaticSolvers/gsStaticNewton.hpp:101-316) ----------------------- */
int klsa_static_create(klsa_problem* prob, const klsa_options* opt, klsa_static** out);
int klsa_static_destroy(klsa_static* s);
int klsa_static_solve(klsa_static* s);                    /* solve(): nonlinear Newton */
int klsa_static_solve_linear(klsa_static* s);             /* solveLinear() */
int klsa_static_set_load_factor(klsa_static* s, double lambda);   /* Residual = lambda*F - Fint */
int klsa_static_set_displacement(klsa_static* s, const double* U);   /* setDisplacement */
int klsa_static_solution(klsa_static* s, double* U);
int klsa_static_iterations(klsa_static* s);

/* ---- arc-length family (gsALMSolvers/gsALMBase.hpp:354-416 and subclasses) ------------
 * method: "Crisfield" (gsALMCrisfield.hpp), "Riks" (gsALMRiks.hpp), "LoadControl"
 * (gsALMLoadControl.hpp), "ConsistentCrisfield" (gsALMConsistentCrisfield.hpp). */
int klsa_alm_create(klsa_problem* prob, const char* method, const klsa_options* opt, klsa_alm** out);
int klsa_alm_destroy(klsa_alm* a);
/* initialize(bool stability) (gsALMBase.h:110-115): with stability != 0 the Jacobian at U is
   computed and factorised and the stability indicator of "BifurcationMethod" evaluated. */
int klsa_alm_initialize(klsa_alm* a, int stability);
/* computeStability(bool jacobian, T shift) (gsALMBase.h:251, gsALMBase.hpp:521-615) -> gsStatus */
int klsa_alm_compute_stability(klsa_alm* a, int jacobian, double shift);
/* indicator() (gsALMBase.h:161), stability() (+1 unstable / -1 stable, gsALMBase.hpp:616-619),
   stabilityChange() (gsALMBase.hpp:624-627) and the number of negative entries of the
   stability vector (inertia of the Jacobian for "Determinant"). Any out pointer may be NULL. */
int klsa_alm_stability(klsa_alm* a, double* indicator, int* stability, int* change, int64_t* negatives);
/* Singular points (gsALMBase.hpp:421-512, 628-852), with the options "SingularPointFailure",
 * "SingularPointTestTol", "SingularPointTestIt", "SingularPointComputeTolE",
 * "SingularPointComputeTolB" (bisection stage when nonzero), "Perturbation" and "Tol".
 * isBifurcation(bool jacobian) (gsALMBase.h:237): 1 bifurcation, 0 limit point, < 0 error.
 * computeSingularPoint(U, L, switchBranch, jacobian, testPoint) (gsALMBase.h:234) -> gsStatus.
 * switchBranch() (gsALMBase.h:257).  solutionV() (gsALMBase.h:169): the null vector. */
int klsa_alm_is_bifurcation(klsa_alm* a, int jacobian);
int klsa_alm_compute_singular_point(klsa_alm* a, const double* U, double L, int switch_branch, int jacobian,
                                    int test_point);
int klsa_alm_switch_branch(klsa_alm* a);
int klsa_alm_solution_v(klsa_alm* a, double* V);
int klsa_alm_step(klsa_alm* a);                           /* step() -> gsStatus */
int klsa_alm_set_length(klsa_alm* a, double length);      /* setLength */
int klsa_alm_reduce_length(klsa_alm* a, double factor);   /* reduceLength */
double klsa_alm_get_length(klsa_alm* a);
int klsa_alm_set_solution(klsa_alm* a, const double* U, double L);      /* setSolution */
int klsa_alm_set_solution_step(klsa_alm* a, const double* DU, double DL); /* setSolutionStep */
int klsa_alm_set_previous(klsa_alm* a, const double* Uprev, double Lprev);  /* setPrevious (gsALMBase.h:185-191) */
/* distance(DeltaU, DeltaL) of Crisfield (gsALMCrisfield.h:79-83) and Riks (gsALMRiks.h:81-84) */
int klsa_alm_distance(klsa_alm* a, const double* DU, double DL, double* out);
int klsa_alm_set_initial_guess(klsa_alm* a, const double* U, double L);  /* setInitialGuess */
int klsa_alm_solution(klsa_alm* a, double* U, double* L);  /* solutionU / solutionL */
/* out: [iterations, residueF, residueU, phi, converged, Lprev, DeltaL_old] */
int klsa_alm_info(klsa_alm* a, double* out);
/* Copies the previous converged point (Uprev, Lprev) and the last step (DeltaUold, DeltaLold). */
int klsa_alm_history(klsa_alm* a, double* Uprev, double* Lprev, double* DUold, double* DLold);

/* ---- learned predictor (no counterpart in the reference; it feeds setInitialGuess,
 * gsALMSolvers/gsALMBase.h:184) ---------------------------------------------------------- */
typedef struct klsa_mlp klsa_mlp;
typedef struct klsa_predictor klsa_predictor;
/* Fully connected n_in -> n_h1 -> n_h2 -> n_out network, GELU, FP32, Glorot init from seed. */
int klsa_mlp_create(int n_in, int n_h1, int n_h2, int n_out, uint64_t seed, klsa_mlp** out);
int klsa_mlp_destroy(klsa_mlp* net);
int64_t klsa_mlp_num_params(const klsa_mlp* net);
int klsa_mlp_get_params(klsa_mlp* net, float* params);       /* W1, b1, W2, b2, W3, b3 (row-major) */
int klsa_mlp_set_params(klsa_mlp* net, const float* params);
int klsa_mlp_forward(klsa_mlp* net, const float* X, int batch, float* Y);
/* MSE loss 1/(2 batch n_out) sum (Y - T)^2 and its gradient (layout of the parameters). */
int klsa_mlp_loss_grad(klsa_mlp* net, const float* X, const float* T, int batch, float* loss, float* grad);
/* Mini-batch Adam (cosine schedule) on the device; final_loss = mean loss of the last epoch. */
int klsa_mlp_train(klsa_mlp* net, const float* X, const float* T, int nsamples, int epochs, int batch, float lr,
                   uint64_t seed, float* final_loss);
/* modes: nmodes x ndof orthonormal basis (public order).  Standardisation vectors of the
 * 4 (nmodes + 1) features and nmodes + 1 targets (NULL: identity).  net may be NULL (plain cubic
 * extrapolation of the last four points). */
int klsa_predictor_create(klsa_problem* prob, klsa_mlp* net, const double* modes, int nmodes,
                          const double* in_mean, const double* in_std, const double* out_mean,
                          const double* out_std, klsa_predictor** out);
int klsa_predictor_destroy(klsa_predictor* pr);
int klsa_predictor_reset(klsa_predictor* pr);
/* Record a converged point (U: ndof, public order) in the predictor's history of four. */
int klsa_predictor_push(klsa_predictor* pr, const double* U, double L);
/* The predicted next point from the last four recorded ones (U: ndof, public order): the value a
 * caller hands to gsALMBase::setInitialGuess (gsALMSolvers/gsALMBase.h:184).  available = 0 (and
 * U, L untouched) while fewer than four points are recorded. */
int klsa_predictor_guess(klsa_predictor* pr, double* U, double* L, int* available);
/* One arc-length point with the learned guess placed as the corrector's start (at most
 * guess_max_iter iterations); on failure the step is redone with the plain tangent predictor.
 * Keeps the predictor's history of converged points.  used_guess (may be NULL) = 1 if the
 * learned guess converged. */
int klsa_alm_step_learned(klsa_alm* a, klsa_predictor* pr, int guess_max_iter, int* used_guess);

/* ---- eigen problems (gsEigenSolvers/gsEigenProblemBase.hpp:152-215) ------------------- */
/* Buckling (gsBucklingSolver.h:127-149): u_L = K_L^-1 (scaling F), B = K(u_L) - K_L,
 * eigenpairs of K_L v = lambda B v by shift-invert Lanczos about ``shift``.
 * values: nev, vectors: nev*ndof (may be NULL). */
int klsa_buckling(klsa_problem* prob, const klsa_options* opt, int nev, double shift, double scaling,
                  double* values, double* vectors);
/* Modal (gsModalSolver.h:46-51): eigenpairs of K v = omega^2 M v about ``shift``. */
int klsa_modal(klsa_problem* prob, const klsa_options* opt, int nev, double shift, double* values,
               double* vectors);
/* gsEigenProblemBase::compute (gsEigenProblemBase.hpp:21-50): every eigenpair of the dense pencil
 * -- kind 0 gsModalSolver (K, M), kind 1 gsBucklingSolver (K_L, K(u_L) - K_L, u_L = K_L^-1 scaling F)
 * -- with the "shift" option applied as A - shift B and added back; eigenvalues ascending,
 * vectors B-normalised.  values: ndof, vectors: ndof x ndof (or NULL).  For dense sizes
 * (at most 4096 dofs); B must be positive definite (else KLSA_SOLVER_ERROR). */
int klsa_eigen_dense(klsa_problem* prob, const klsa_options* opt, int kind, double scaling, double* values,
                     double* vectors);
/* gsEigenProblemBase::computePower (gsEigenProblemBase.hpp:218-258): the eigenpair of smallest
 * |lambda| by power iteration on A^-1 B from the all-ones vector ("tolerance" option, at most 100
 * steps, KLSA_NOT_CONVERGED after the last).  value: 1, vector: ndof (Euclidean-normalised) or NULL. */
int klsa_eigen_power(klsa_problem* prob, const klsa_options* opt, int kind, double scaling, double* value,
                     double* vector);

/* ---- adaptive parallel arc-length method (gsALMSolvers/gsAPALM.hpp, gsAPALMData.hpp) -----
 * Over an arc-length object of method Crisfield or Riks (the methods with a distance).  The jobs
 * run in queue order on the device solver: the schedule of a one-process reference run.  Options:
 * "MaxIt" (1000), "SubIntervals" (2), "SingularPoint" (0), "BranchLengthMultiplier" (1),
 * "BifLengthMultiplier" (0.1), and the data options "MaxLevel" (5) and "Tolerance" (0.1). */
typedef struct klsa_apalm klsa_apalm;
int klsa_apalm_create(klsa_alm* alm, const klsa_options* opt, klsa_apalm** out);
int klsa_apalm_destroy(klsa_apalm* ap);
int klsa_apalm_initialize(klsa_apalm* ap);                           /* initialize(): start at (0, 0) */
int klsa_apalm_add_start(klsa_apalm* ap, const double* U, double L, double dL);   /* _initStart */
int klsa_apalm_serial_solve(klsa_apalm* ap, int nsteps);             /* serialSolve(Nsteps) */
/* Another solver for parallelSolve's interval corrections -- the reference's MPI workers
 * (gsAPALM.hpp:276-378) as concurrent solvers on one GPU.  worker: an arc-length object of the
 * same method and options on its own problem made from the same description.  With W solvers
 * parallelSolve hands a job to every idle one, submits the oldest job handed out when it is
 * done and refills its solver at once (the MPI schedule, jobs finishing in the order they were
 * handed out); each solver runs on its own stream from its own host thread. */
int klsa_apalm_add_worker(klsa_apalm* ap, klsa_alm* worker);
int klsa_apalm_parallel_solve(klsa_apalm* ap);                       /* parallelSolve() */
int klsa_apalm_solve(klsa_apalm* ap, int nsteps);                    /* solve(Nsteps) */
int klsa_apalm_branches(klsa_apalm* ap);
int klsa_apalm_solutions(klsa_apalm* ap, int branch);                /* points of getFlatSolutions(branch) */
/* point k of branch b: U (public order, may be NULL), L, curve time (getFlatTimes), level (getFlatLevels) */
int klsa_apalm_solution(klsa_apalm* ap, int branch, int k, double* U, double* L, double* time, int* level);

/* ---- time integrators (gsDynamicSolvers/gsDynamicBase.h:185-260 and the integrators) ----
 * method: "Newmark" (gsDynamicNewmark.hpp), "Bathe" (gsDynamicBathe.hpp), "Wilson"
 * (gsDynamicWilson.hpp), "ExplicitEuler" (gsDynamicExplicitEuler.hpp), "ImplicitEuler"
 * (gsDynamicImplicitEuler.hpp), "RK4" (gsDynamicRK4.hpp).  nonlinear selects the reference's
 * _NL template flag: 1 = tangent K(U) and residual R(U,t) = f(t) F - Fint(U) (the Mass,
 * Damping, Jacobian, TResidual constructor), 0 = constant stiffness K_L and force f(t) F (the
 * Mass, Damping, Stiffness, TForce constructor).  M is the consistent mass.  Options: "DT" (1e-2),
 * "MaxIter" (100), "TolF" (1e-3), "TolU" (1e-6), "Quasi" (0), "QuasiIterations" (1), "alpha",
 * "delta", "gamma" (Newmark 0.25/0.5, Bathe 0.25/0.5/0.5, Wilson 0.25/0.5/1.4), "Solver"
 * (a direct solver: SimplicialLDLT), plus, without a reference key, "DampingMass" and
 * "DampingStiffness" (Rayleigh damping C = cM M + cK K_L; the reference takes C from a Damping_t
 * callback, zero in its tutorials) and "FrontPrecision" (64, or 32 with FP64 refinement).
 * ImplicitEuler solves its block system exactly where the reference runs GMRES on it. */
typedef struct klsa_dynamic klsa_dynamic;
int klsa_dynamic_create(klsa_problem* prob, const char* method, int nonlinear, const klsa_options* opt,
                        klsa_dynamic** out);
int klsa_dynamic_destroy(klsa_dynamic* d);
/* Load factor f(t): piecewise linear through (t[i], f[i]), t non-decreasing, constant beyond the
 * ends; n = 0 restores f = 1 (the TForce_t / TResidual_t callbacks of the reference). */
int klsa_dynamic_set_load_table(klsa_dynamic* d, const double* t, const double* f, int n);
/* setU / setV / setA and solutionU / solutionV / solutionA (public free-dof order; a NULL
 * pointer leaves that field unchanged / unread). */
int klsa_dynamic_set_state(klsa_dynamic* d, const double* U, const double* V, const double* A);
int klsa_dynamic_state(klsa_dynamic* d, double* U, double* V, double* A);
/* step(dt) (gsDynamicBase.h:196-208), dt <= 0: the "DT" option.  Returns the gsStatus of the step;
 * the time advances by dt in every case. */
int klsa_dynamic_step(klsa_dynamic* d, double dt);
int klsa_dynamic_set_time(klsa_dynamic* d, double t);
double klsa_dynamic_time(klsa_dynamic* d);
/* Newton iterations of the last step (1 for the explicit and linear integrators) */
int klsa_dynamic_iterations(klsa_dynamic* d);

/* ---- batched Newton solves of many patches (no counterpart in the reference) ------------
 * Equivalent to one gsStaticNewton::solve() per instance (gsStaticNewton.hpp:101-193), each
 * with its own assembler; here all instances share every launch: a persistent assembly kernel
 * over the elements of all instances, one multifrontal factorisation of the merged
 * block-diagonal tangent (an elimination forest), device-side convergence control and one
 * CUDA graph per Newton iteration.  Instances: degree 2 or 3. */
typedef struct klsa_batch klsa_batch;
typedef struct klsa_batch_newton klsa_batch_newton;
int klsa_batch_create(const klsa_patch_desc* descs, int n, klsa_batch** out);
int klsa_batch_destroy(klsa_batch* b);
/* out[4]: instances, free dofs (all instances), CSR nonzeros (all instances), front pool bytes */
int klsa_batch_info(klsa_batch* b, double* out);
/* free dofs of instance i (its public order, as klsa_problem_ndof) */
int64_t klsa_batch_instance_ndof(klsa_batch* b, int i);
/* Times the launch shapes of the persistent assembly kernels and keeps the fastest.  log:
 * (kind 0 tangent / 1 internal force, degree, blocks per SM, ms) per trial, up to cap rows;
 * returns the number of rows. */
int klsa_batch_autotune(klsa_batch* b, double* log, int cap);
/* Options as gsStaticNewton ("tol", "tolF", "tolU", "maxIt", "Relaxation") plus "LoadFactor" and
 * "Refinement" (sweeps of iterative refinement of each Newton step against the assembled
 * tangent, default 1). */
int klsa_batch_newton_create(klsa_batch* b, const klsa_options* opt, klsa_batch_newton** out);
int klsa_batch_newton_destroy(klsa_batch_newton* s);
/* solve() of every instance -> Success when all converged, else NotConverged; per-instance
 * statuses (gsStatus) and iteration counts from klsa_batch_newton_results. */
int klsa_batch_newton_solve(klsa_batch_newton* s);
int klsa_batch_newton_reset(klsa_batch_newton* s);   /* U = 0, next solve() starts linearly */
int klsa_batch_newton_results(klsa_batch_newton* s, int* status, int* iterations);
int klsa_batch_newton_solution(klsa_batch_newton* s, int i, double* U);   /* public order */
int klsa_batch_sync(klsa_batch* b);
int klsa_batch_event_record(klsa_batch* b, int slot);
int klsa_batch_event_elapsed(klsa_batch* b, int slot_a, int slot_b, float* ms);

/* ---- measurement helpers (no counterpart in the reference, which has no device) -------- */
/* Per-phase device times from CUDA events on the problem streams: ms[8], counts[8] for
 * 0 tangent assembly, 1 factorisation, 2 solves, 3 residual, 4/5/6 multifrontal update /
 * diagonal / panel launches, 7 other. */
int klsa_profile_enable(int on);
int klsa_profile_read(double* ms, uint64_t* counts);
int klsa_profile_reset(void);
/* Records CUDA event `slot` (0..15) on the problem's stream; elapsed time between two slots. */
int klsa_event_record(klsa_problem* prob, int slot);
int klsa_event_elapsed(klsa_problem* prob, int slot_a, int slot_b, float* ms);
int klsa_problem_sync(klsa_problem* prob);
/* out[18]: ndof, nnz, elements, Gauss points, front pool bytes, factorisation flops,
 * tangent-assembly flops, multifrontal tree nodes, algorithmic bytes per factorisation of the
 * diagonal / panel / update kernels (3), their flops (3), their launches per factorisation (3),
 * bytes of one triangular solve */
int klsa_problem_stats(klsa_problem* prob, double* out);

/* ---- host-only symbolic queries (no device call) -------------------------------------- */
int klsa_nd_stats(int n1, int n2, int p, const uint8_t* fixed, int leaf_max, double* out);
int klsa_nd_export(int n1, int n2, int p, const uint8_t* fixed, int leaf_max, int32_t* full2int,
                   int32_t* node_info, int32_t* halo_ids, int64_t capacity_nodes, int64_t capacity_halo);

#ifdef __cplusplus
}
#endif

#endif /* KLSHELL_GB300_H */
