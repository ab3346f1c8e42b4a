/* spde_gb300: GB300-native inference hot path of spdepy (C ABI).
 *
 * Every entry point returns an int status (SPDE_OK = 0), never throws, and runs
 * on the plan's CUDA stream (the default stream unless spde_plan_set_stream is
 * called).  Arrays documented as "device" are CUDA device pointers owned by the
 * caller; "host" arrays are ordinary host memory.  A plan is not thread-safe:
 * use one plan per host thread.
 *
 * Node numbering is the reference's: node k = t*Mx*Ny + j*Mx + i for cell
 * (i, j) at time t (spdes/advection_diffusion2D.py:112-116), on the grid
 * including any extension cells.  "Stencil layout" stores nslots values per
 * node (43 for T > 1: 9 at t-1, 25 at t, 9 at t+1; 25 for T == 1), slot order
 * dt-major, then dy, then dx, each ascending.
 */
#ifndef SPDE_GB300_H
#define SPDE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPDE_OK 0
#define SPDE_ERR_ARG 1
#define SPDE_ERR_CUDA 2
#define SPDE_ERR_NOT_SPD 3
#define SPDE_ERR_NO_MEMORY 4
#define SPDE_ERR_STATE 5
#define SPDE_ERR_NOT_CONVERGED 6

#define SPDE_PRECISION_FP64 0 /* factor, solves and inverse in FP64 */
#define SPDE_PRECISION_MIXED 1 /* FP32 factor, FP64 pivots / log-det / refinement */
#define SPDE_PRECISION_ITERATIVE 2 /* no factorisation: assembly, products, PCG */

#define SPDE_PRECOND_NONE 0
#define SPDE_PRECOND_JACOBI 1
#define SPDE_PRECOND_LEARNED 2
#define SPDE_PRECOND_LEARNED_COMPACT 3 /* learned, weights from spde_precond_weights_compact */
#define SPDE_PRECOND_IC0 4 /* incomplete Cholesky, zero fill, natural order (spde_pcg only) */
#define SPDE_PRECOND_NPARAMS 3323

typedef struct SpdePlan SpdePlan;

typedef struct {
  int64_t n;            /* nodes */
  int64_t nfronts;      /* dense fronts (tree nodes of the dissection) */
  int32_t max_depth;
  int32_t max_front;    /* largest front order */
  int32_t nslots;
  int32_t precision;
  double factor_flops;  /* algorithmic flops of one factorisation */
  double selinv_flops;  /* algorithmic flops of one selected inversion */
  double nnz_l;         /* entries of the dense-front factor */
  double bytes_factor;  /* device bytes of the factor arena */
  double bytes_work;    /* device bytes of the update / inverse pools */
  int64_t launches;     /* kernel launches issued by this plan so far */
} SpdePlanInfo;

/* Model description (spde_set_model).  Canonical parameter vector theta:
 *   [0,nk) log kappa | [nk,2nk) log gamma | [2nk,3nk) vx | [3nk,4nk) vy |
 *   [4nk,4nk+nw) advection | log sigma | log kappa0, log gamma0, vx0, vy0 | log tau
 * with nk = nbasis if var_h else 1 and nw = 2 (constant velocity), 2*nbasis
 * (B-spline velocity), 1 (lambda times a given field) or 0 (spatial model).
 * The last five entries before log tau describe the initial-field
 * Whittle-Matern model of spatio-temporal models and are ignored when T == 1.
 * Separable models Q = Qt (x) Qs (spdes/seperable_spatial_temporal{,_ha,
 * _idiffusion}2D.py) use the spatial layout (adv = 0, Qs = A^T V^-1 A with
 * A = V kappa - A_H) and put their temporal parameters in the log sigma slot
 * (log rho, or a) and the log kappa0 slot (log sigma of the (a, sigma) form). */
typedef struct {
  int32_t Mx, Ny, T;
  int32_t bc;           /* 1: Neumann (zero flux), 3: Dirichlet (zero) */
  double hx, hy, dt;
  int32_t diff_form;    /* 0: gamma I, 1: gamma I + v v^T, 2: half-angle */
  int32_t var_h;        /* 0: constant kappa/gamma/v; 1: B-spline fields */
  int32_t adv;          /* 0 none, 1 constant, 2 B-spline field, 3 lambda * given field */
  int32_t nbasis;       /* B-spline functions (Nbs^2) */
  const double* bs;     /* host, Ns x nbasis, cell centres            (var_h) */
  const double* bsH;    /* host, Ns x 4 x nbasis, faces W,E,S,N        (var_h) */
  const double* bsA;    /* host, Ns x 4 x nbasis, faces E,N,W,S        (adv == 2) */
  const double* ww;     /* host, Ns x 4 given face velocities          (adv == 3) */
  int32_t mod0_diff_form;
  int32_t mod0_bc;
  int32_t temporal;     /* separable plans only: 1 AR(1) in log rho, 2 (a, log sigma); 0 otherwise */
} SpdeModelDesc;

/* ---- B3: stencil triplets.  Replace the ctypes calls
 * AH_new/AH_Row/AH_Col/AH_Val/AH_delete (spdes/ccode/AcH_2D_b1.cpp:170-185,
 * AH_2D_b1.cpp:154-169) and Aw_new/Aw_Row/Aw_Col/Aw_Val/Aw_delete
 * (Acw_2D_b1.cpp:117-132, Aw_2D_b1.cpp:136-151).  Outputs are device arrays of
 * 9*M*N (diffusion) or 5*M*N (advection) triplets with the reference's
 * row == M*N sentinel; values match the reference's doubles bit for bit.
 * field = 0: H is one 2x2 (row-major) / G is (wx, wy); field = 1: H is
 * (M*N, 4, 2, 2) / G and dG are (M*N, 4).  Unlike the reference, inputs are
 * never modified.  bc must be 1 or 3. */
int spde_diffusion_triplets(int M, int N, const double* H, int field, double hx, double hy, int bc, int* row,
                            int* col, double* val, void* stream);
int spde_advection_triplets(int M, int N, const double* G, const double* dG, int field, double hx, double hy, int bc,
                            int diff, int* row, int* col, double* val, void* stream);

/* ---- plan: symbolic analysis + device arenas (the analysis half of
 * sksparse.cholmod.cholesky, called at spdes/advection_diffusion2D.py:117,193).
 * precision SPDE_PRECISION_ITERATIVE makes a plan without ordering or factor
 * arenas (assembly, products and PCG only); factor-based calls then return
 * SPDE_ERR_STATE. */
int spde_plan_create(int Mx, int Ny, int T, int precision, int leaf_max, SpdePlan** out);
/* Plan for separable space-time models Q = Qt (x) Qs (the reference's
 * SeperableSpatialTemporal{,Ha,IDiffusion}2D, spdes/seperable_spatial_temporal2D.py:
 * 64-83): every time slice couples to its neighbours through the 25-point Qs, a
 * 75-slot stencil.  T >= 2; precision FP64 or mixed.  The learned preconditioner
 * and spde_qsqrt return SPDE_ERR_STATE on such plans. */
int spde_plan_create_separable(int Mx, int Ny, int T, int precision, int leaf_max, SpdePlan** out);
int spde_plan_destroy(SpdePlan* plan);
int spde_plan_set_stream(SpdePlan* plan, void* stream);
int spde_plan_info(const SpdePlan* plan, SpdePlanInfo* info);
const char* spde_last_error(const SpdePlan* plan);
/* Optional per-launch timing with CUDA events on the plan's stream (no
 * reference counterpart; measurement only): enable 1 times every launch, 2 only
 * the tensor-core products, 0 none.  read_profile fills 10 entries per
 * launch class (0 memset, 1 extend-add, 2 diagonal block, 3 tiled product on
 * the CUDA cores, 4 forward gather, 5 backward gather, 6 inverse gather,
 * 7 transpose, 8 inverse extraction, 9 tiled product on the tensor cores):
 * milliseconds, algorithmic flops, launches. */
int spde_plan_set_profiling(SpdePlan* plan, int enable);
int spde_plan_read_profile(SpdePlan* plan, double* ms, double* flops, int64_t* count, int reset);
/* The same timing split by call site of the tiled product (18 entries: factor
 * panel solve / panel update / Schur update, solve steps, inverse steps). */
int spde_plan_read_sites(SpdePlan* plan, double* ms, double* flops, int64_t* tiles, int reset);
/* Concurrency of spde_loglike (no reference counterpart): with 2 pipelines (the
 * default) Q + tau S^T S is factored, solved and inverted on a second set of
 * arenas with its own host thread while Q runs on the plan's own, so the two
 * factorisations' latency-bound top levels overlap; it doubles the factor and
 * inverse memory.  Each pipeline then runs its factorisation and solve on a
 * greatest-priority stream and its inversion on a least-priority stream of the
 * plan, ordered after the work already on the plan's stream and joined back to
 * it before spde_loglike returns.  1 runs them one after the other on the plan's
 * stream and one set of arenas. */
int spde_plan_set_pipelines(SpdePlan* plan, int pipelines);
/* Failure detection (no reference counterpart): every wait inside the
 * tensor-core kernels, and every wait of the one-right-hand-side triangular
 * sweeps on another block's completion flag, gives up after this many
 * nanoseconds of wall clock (0 restores the default, 2 s); the kernel then
 * records an error (the tensor-core kernels wait for their issued tensor-core
 * work and free their tensor memory first) and returns, and the factorisation,
 * inversion, solve or sample returns SPDE_ERR_CUDA with the plan still usable.
 * Tests lower the limit to make the waits run out. */
int spde_plan_set_wait_limit(SpdePlan* plan, int64_t ns);
/* Symbolic analysis without a GPU (host only): statistics and the ordering. */
int spde_symbolic_info(int Mx, int Ny, int T, int leaf_max, SpdePlanInfo* info);
int spde_symbolic_export(int Mx, int Ny, int T, int leaf_max, int32_t* perm, int32_t* front_ns, int32_t* front_nb,
                         int32_t* front_parent, int64_t nfronts_cap);

/* ---- assembly: makeQ (spdes/advection_diffusion2D.py:86-117,
 * spdes/var_advection_var_diffusion2D.py:83-116,
 * spdes/whittle_matern_anisotropic2D.py:59-75). */
int spde_set_model(SpdePlan* plan, const SpdeModelDesc* desc);
int spde_assemble(SpdePlan* plan, const double* theta_host, int ntheta);
/* Q (+ tau S^T S when with_obs) in stencil layout, natural order, device FP64. */
int spde_export_q(SpdePlan* plan, int with_obs, double tau, double* q_dev);
/* y = (Q [+ tau S^T S]) x, natural order, nrhs columns row-major, device FP64. */
int spde_spmv(SpdePlan* plan, int with_obs, double tau, const double* x_dev, double* y_dev, int nrhs);

/* ---- observations: S = selected identity rows (grids/spat2Dtemp_regular_mesh.py:35-58);
 * idx are node indices (duplicates allowed), host int64. */
int spde_set_obs(SpdePlan* plan, const int64_t* idx_host, int m);
/* The same with a weight per observation (host FP64, finite, >= 0): the
 * matrices "with observations" become Q + tau sum_i w_i e_{idx_i} e_{idx_i}^T.
 * Model.update accumulates Q += tau_k S_k^T S_k over calls whose tau_k differ
 * (model.py:120-127): weights tau_k with tau = 1 give that sum.  spde_loglike
 * and the conditional-mean right-hand sides treat every observation alike and
 * are meant for unweighted sets. */
int spde_set_obs_weighted(SpdePlan* plan, const int64_t* idx_host, const double* weights_host, int m);

/* ---- factorisation: cholesky(Q) / cholesky(Q + tau S^T S) and Factor.logdet()
 * (spdes/advection_diffusion2D.py:117,192-193,198). */
int spde_factor(SpdePlan* plan, int with_obs, double tau, double* logdet);
/* Factor.solve_A (spdes/advection_diffusion2D.py:194,201-202; model.py:126):
 * x = A^-1 b for the factored matrix, device FP64, natural order, nrhs columns
 * row-major; refine_iters FP64 iterative-refinement steps (stop at rel. residual
 * <= tol); *resid receives the final relative residual. */
int spde_solve(SpdePlan* plan, const double* b_dev, double* x_dev, int nrhs, int refine_iters, double tol,
               double* resid);
/* Factor.apply_Pt(Factor.solve_Lt(z)) (model.py:80): x = P L^-T z for the factored
 * matrix; z, x device FP64 natural order (nrhs columns).  With Q = P L L^T P^T the
 * columns of x are draws from N(0, Q^-1) when z ~ N(0, I). */
int spde_sample(SpdePlan* plan, const double* z_dev, double* x_dev, int nrhs);
/* Selected inverse (rqinv.R:18-205 via model.py:89-118): Z = A^-1 on the stencil
 * pattern, stencil layout, device FP64.  Consumes the factor. */
int spde_selinv(SpdePlan* plan, double* zq_dev);
/* d/dtheta <Gbar, Q(theta)> for a symmetric Gbar in stencil layout (device
 * FP64); grad_host receives ntheta-1 values (all but log tau). */
int spde_adjoint(SpdePlan* plan, const double* gbar_dev, double* grad_host);
/* The same gradient without any device allocation (no reference counterpart).
 * For callers that cannot call cudaMalloc during the computation, e.g. code
 * that runs under a framework owning all device memory through its own pool,
 * or code that must not synchronise the device mid-stream (cudaMalloc and
 * cudaFree can).  The caller passes Gbar and receives ntheta-1 values in
 * grad_dev (both device FP64); the work array is a fixed 8 MiB static device
 * array, enough for grids with Mx*Ny <= 9892 cells (larger grids return
 * SPDE_ERR_ARG).  The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress); make that first call before any stream
 * capture.  All calls share the one array: calls that overlap on the GPU
 * (other streams, other host threads, other plans) race on it.  Unlike
 * spde_adjoint, the call only enqueues the work on the plan's stream (on the
 * plan's device, whichever device is current) and returns before the gradient
 * is written: gbar_dev must be ready on that stream, and grad_dev is valid once
 * the stream has reached this point (e.g. after cudaStreamSynchronize). */
int spde_adjoint_noalloc(SpdePlan* plan, const double* gbar_dev, double* grad_dev);

/* ---- log-likelihood and gradient: logLike (spdes/advection_diffusion2D.py:187-223).
 * y_dev: m x r observations (device FP64, row-major, in spde_set_obs order).
 * grad_mode: 0 none, 1 exact traces by selected inversion, 2 Hutchinson with the
 * n x nh1 probe matrix probes_dev (device FP64 entries +-1).  Outputs the
 * reference's normalised objective f = -like/(m r) and jac = -g/(m r) (ntheta
 * values, canonical order). */
int spde_loglike(SpdePlan* plan, const double* theta_host, int ntheta, const double* y_dev, int r, int grad_mode,
                 const double* probes_dev, int nh1, double* f, double* jac_host);
/* Conditional mean mu = mu0 + tau (Q + tau S^T S)^-1 S^T (y - S mu0) (model.py:120-127);
 * y_dev m values, mu0_dev/mu_dev n values (device FP64). */
int spde_conditional_mean(SpdePlan* plan, double tau, const double* y_dev, const double* mu0_dev, double* mu_dev);

/* ---- learned preconditioner and PCG (no reference counterpart: the reference
 * factors every system with CHOLMOD; these serve grids too large to factor).
 * M^-1 = G^T G with G a 27-point space-time stencil whose weights a small
 * network computes from each node's normalised row of A = Q (+ tau S^T S).
 * Network parameters: SPDE_PRECOND_NPARAMS FP32 values in device memory
 * (layout W1[32][42], b1[32], W2[32][32], b2[32], W3[27][32], b3[27]). */
int spde_precond_nparams(void);
/* G weights (27 x n, offset-major: weight of offset o = (dt+1) 9 + (dy+1) 3 +
 * (dx+1) at node p in w_dev[o n + p]; FP32, device) for the assembled model; act_dev (optional,
 * n x 107 FP32) keeps the activations a gradient step needs. */
int spde_precond_weights(SpdePlan* plan, int with_obs, double tau, const float* params_dev, float* w_dev,
                         float* act_dev);
/* The same operator G with its rows stored once per (spatial cell, time class)
 * plus once per distinct observed node: Q's stencil coefficients do not depend
 * on time, so a node's row of A (and the network output) depends on its time
 * step only through the classes first / interior / last step, unless the node
 * is observed.  The compact array (FP32, device) has
 * spde_precond_compact_size() values: a 4-value header, then 27 (3 Mx Ny +
 * distinct observed nodes); it stays in L2 where per-node weights (27 n) would
 * stream from HBM on every application.  Use it with
 * SPDE_PRECOND_LEARNED_COMPACT, the same with_obs and the same observation set
 * (a solve checks the header and returns SPDE_ERR_STATE otherwise). */
int spde_precond_compact_size(const SpdePlan* plan, int64_t* nfloats);
int spde_precond_weights_compact(SpdePlan* plan, int with_obs, double tau, const float* params_dev, float* w_dev);
/* Training loss ||z - G A G^T z||^2 / (n k) for the probe block z_dev (n x k,
 * row-major, FP64) and its gradient with respect to the parameters (grad_dev,
 * SPDE_PRECOND_NPARAMS FP32). */
int spde_precond_grad(SpdePlan* plan, int with_obs, double tau, const float* params_dev, const float* w_dev,
                      const float* act_dev, const double* z_dev, int k, double* loss, float* grad_dev);
/* One Adam update of n parameters on the plan's stream (step t >= 1). */
int spde_adam_step(SpdePlan* plan, float* params_dev, const float* grad_dev, float* m_dev, float* v_dev, int n,
                   double lr, double b1, double b2, double eps, int t);
/* Square root of the prior precision, Q = B^T B (no reference counterpart; the
 * time-block structure of spdes/advection_diffusion2D.py:101-116 written as a
 * sum of squares): y = B x (transpose 0) or B^T x (transpose 1), n x nrhs
 * row-major, device FP64.  B^T eps with eps ~ N(0, I) has covariance Q, which
 * gives posterior draws by one PCG solve (Model.sample without a factor). */
int spde_qsqrt(SpdePlan* plan, int transpose, const double* x_dev, double* y_dev, int nrhs);
/* z <- (I - omega D^-1 A)^sweeps z, then every column scaled to unit RMS
 * (z_dev n x nrhs, FP64): the error a damped-Jacobi sweep leaves after
 * `sweeps` steps from z, i.e. the smooth residual directions CG has to work on;
 * used as training probes. */
int spde_jacobi_smooth(SpdePlan* plan, int with_obs, double tau, double omega, int sweeps, double* z_dev, int nrhs);
/* x = A^-1 b by preconditioned CG (x from 0), nrhs columns row-major, FP64
 * device; precond SPDE_PRECOND_* (w_dev: G weights for LEARNED, compact weights
 * for LEARNED_COMPACT).  The iterations run in FP32 (stencil product, vectors,
 * preconditioner; IC0 factors A in FP32 on entry, level-scheduled on the
 * lattice, with a diagonal shift raised until no pivot breaks down); the
 * solution is accumulated in FP64 and the residual
 * replaced by the true FP64 residual b - A x whenever the recursive one has
 * fallen tenfold (and every 64 iterations).  Stops when every column's true
 * residual reaches ||b - A x|| <= tol ||b|| or after maxit iterations; *relres
 * is the worst true relative residual.  Returns SPDE_ERR_NOT_CONVERGED when the
 * tolerance was not reached. */
int spde_pcg(SpdePlan* plan, int with_obs, double tau, int precond, const float* w_dev, const double* b_dev,
             double* x_dev, int nrhs, double tol, int maxit, int* iters, double* relres);

/* Gradient of the objective (spde_loglike's jac, canonical order) for the model
 * last assembled with log tau = log(tau), on grids too large to factor:
 * Hutchinson traces (the reference's estimator, advection_diffusion2D.py:200-209)
 * with the nh1 probe columns probes_dev (n x nh1, +-1, device FP64), every solve
 * by PCG (precond SPDE_PRECOND_*; w_q_dev / w_qc_dev: G weights for Q and for
 * Q + tau S^T S) to relative residual tol.  The objective itself needs
 * log-determinants and is not computed.  *iters receives the PCG iterations
 * summed over the three solves. */
int spde_loglike_grad_pcg(SpdePlan* plan, double tau, const double* y_dev, int r, const double* probes_dev, int nh1,
                          int precond, const float* w_q_dev, const float* w_qc_dev, double tol, int maxit,
                          double* jac_host, int* iters);

#ifdef __cplusplus
}
#endif
#endif /* SPDE_GB300_H */
