/*
 * picuda.h -- C ABI of libpicuda.so, the GB300 (sm_103a) backend for the matrix-free
 * Schur-block Liouvillian of PermutationalInvariantDynamics.jl and the Krylov solvers
 * wrapped around it.
 *
 * The reference package has no native FFI; each entry point below names the Julia
 * function whose work it replaces (paths are inside the reference project).  A Julia
 * extension binds these with `ccall` behind `compile(model; backend=:cuda)`,
 * `apply!`, `solve_dynamics(...; algorithm=ExpvAlgorithm(...))` and
 * `stationary_state(...; algorithm=GMRESAlgorithm(...))`.
 *
 * Conventions
 *  - Every function returns PI_OK (0) or a negative status; pi_last_error() gives the
 *    message of the last failure on the calling thread.
 *  - Complex vectors are interleaved (re, im) arrays in the reference's coordinate order:
 *    sectors in descending partition order (basis.jl:27), column-major n x n blocks
 *    (basis.jl:31, :90-93), GT patterns in ascending entry order (gtpatterns.jl:92-106).
 *  - "dev" pointers are device pointers; "host" pointers are ordinary host memory.
 *  - Sector offsets reported by this ABI are 0-based (the Julia basis stores 1-based).
 */
#ifndef PICUDA_H
#define PICUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PI_OK 0
#define PI_ERR_INVALID_ARGUMENT (-1)   /* maps to ArgumentError */
#define PI_ERR_DIMENSION (-2)          /* maps to DimensionMismatch */
#define PI_ERR_OUT_OF_MEMORY (-3)
#define PI_ERR_NOT_CONVERGED (-4)      /* krylov.jl:873, krylov_extensions.jl:1559-1561 */
#define PI_ERR_CUDA (-5)
#define PI_ERR_UNSUPPORTED (-6)        /* model outside the CUDA backend (d != 2, p-body, ...) */
#define PI_ERR_NO_DEVICE (-7)
#define PI_ERR_BUSY (-8)               /* a plan in use (PI_CONCURRENCY_REJECT) */

/* Term kinds (terms.jl:118-149). Operators are 2x2 complex, column-major interleaved. */
#define PI_TERM_HAMILTONIAN 0      /* CollectiveHamiltonian / LocalHamiltonian: rate/hbar */
#define PI_TERM_LOCAL_JUMP 1       /* LocalJump: rate * sum_i D[L_i] */
#define PI_TERM_COLLECTIVE_JUMP 2  /* CollectiveJump: rate * D[sum_i L_i] */

/* Precision of an apply or solve. */
#define PI_FP64 0  /* plain complex FP64 in reference coordinates */
#define PI_FP32 1  /* complex FP32 applies; solver accuracy restored in FP64 */

/* Coordinates of an FP32 vector. */
#define PI_COORDS_REFERENCE 0   /* the reference's PI coefficients x */
#define PI_COORDS_POPULATION 1  /* population coordinates z = sqrt(f^nu) x per sector */

typedef struct pi_plan pi_plan;

/* ---- library / device -------------------------------------------------------------- */

/* Message of the last failing call on this thread (accelerators.jl:348-350 reasons). */
int pi_last_error(char* buf, size_t len);

/* Capability report; replaces _accelerator_extension_capability(::Val{:cuda})
 * (accelerators.jl:41).  functional = 1 only after a device query succeeded. */
typedef struct {
  int functional;
  int supports_matrixfree_pi;
  int device_count;
  int sm_count;
  int cc_major, cc_minor;
  size_t total_memory;
  char device_name[128];
} pi_capability_t;
int pi_capability(pi_capability_t* out);

/* ---- plan: compile(model; backend=:cuda) -------------------------------------------- */

/* Builds and uploads the fused plan of a qubit model; replaces compile (liouvillian.jl:
 * 4040-4098) -> LiouvillianPlan (:1844-1851) -> compile_term (:1290-1371) and the fusion
 * (:1700-1738).  sector_ks lists the retained sectors (N-k, k) (NULL = all); ops holds
 * nterms 2x2 column-major interleaved complex matrices (8 doubles each); hbar may be NULL
 * (all ones).  The plan owns its device tables and a CUDA stream. */
int pi_plan_create(int N, int d, int nsectors, const int* sector_ks, int nterms,
                   const int* term_kind, const double* ops, const double* rates,
                   const double* hbar, pi_plan** out);
int pi_plan_destroy(pi_plan* plan);

/* The adjoint generator as a plan of its own: the conjugate transpose of the PI-coordinate
 * matrix, the operator of apply_adjoint! (liouvillian.jl:3107-3143, 3275-3324,
 * 4190-4266).  Built on the host from plan's lowered stencil (every term transposed:
 * sectors swapped, offsets negated, coefficients conjugated and shifted), so every apply
 * and solver entry point runs it; destroy it with pi_plan_destroy. */
int pi_plan_adjoint(const pi_plan* plan, pi_plan** out);

/* Concurrent calls on one plan (solves, Arnoldi, RK4, host-buffer applies: every call that
 * uses the plan's own stream, staging buffers or engine).  PI_CONCURRENCY_WAIT (the default)
 * serializes them: a second host thread waits for the first, as the reference's locked
 * MatrixFreeLiouvillian does for shared tasks (liouvillian.jl:35-60).  PI_CONCURRENCY_REJECT
 * makes a call that finds the plan in use return PI_ERR_BUSY at once, the rule of the
 * reference's per-task workspaces (threaded_apply.jl:575).  The device-pointer applies
 * (pi_apply_f64, pi_apply_f32, pi_apply_f32_em) only read the plan and run on the caller's
 * stream, so they never wait. */
#define PI_CONCURRENCY_WAIT 0
#define PI_CONCURRENCY_REJECT 1
int pi_plan_set_concurrency(pi_plan* plan, int mode);

typedef struct {
  int N;
  int nsectors;
  long long dim;     /* length(basis) = sum n^2 (basis.jl:35) */
  int max_block;     /* largest block dimension */
  int max_terms;     /* stencil terms of the busiest sector */
  long long stencil_terms; /* total stencil terms over all sectors */
  size_t device_bytes;     /* device memory owned by the plan tables */
  int batched_kernel;      /* applies with >= 2 columns: 0 general tile kernel, 1 fixed-structure
                              register kernel, 2 canonical-position register-reuse kernel */
} pi_plan_info_t;
int pi_plan_info(const pi_plan* plan, pi_plan_info_t* out);

/* Bit-exact basis maps (basis.jl:20-34): k values, 0-based offsets and block sizes of
 * every sector, each array of length nsectors. */
int pi_plan_sectors(const pi_plan* plan, int* ks, long long* offsets, int* dims);
/* GT patterns of one sector as entry triples {m, lam1, lam2} in in-block order
 * (gtpatterns.jl:92-106); entries has room for 3*n ints. */
int pi_plan_gt_patterns(const pi_plan* plan, int sector, int* entries);
/* Trace functional: sqrt(f^nu) on every block diagonal (source_protocol.jl:15-34).
 * idx/vals have room for sum_s n_s entries. */
int pi_plan_trace_functional(const pi_plan* plan, long long* idx, double* vals);
/* Per-sector sqrt(f^nu) (the population scaling of the FP32 coordinates). */
int pi_plan_sector_scales(const pi_plan* plan, double* sqrt_f);

/* ---- host-only inspection of the lowering (no device needed) ----------------------- */

/* Exports the stencil tables that pi_plan_create would upload, for the same arguments.
 * Two-call pattern: with term_table and coef NULL it only writes counts[0] = number of
 * stencil terms and counts[1] = number of complex coefficients.  term_table receives 8
 * ints per term {out_sector, src_sector, kind, cls, dr, dc, alpha_off, beta_off} (kind 0
 * ADD (alpha[a]+beta[b]) x[a,b], 1 LEFT alpha[a] x[a+dr,b], 2 RIGHT beta[b] x[a,b+dc],
 * 3 SAND alpha[a] beta[b] x[a+dr,b+dc]; offsets -1 when unused) and coef the interleaved
 * complex FP64 coefficient pool in reference coordinates. */
int pi_stencil_export(int N, int d, int nsectors, const int* sector_ks, int nterms,
                      const int* term_kind, const double* ops, const double* rates,
                      const double* hbar, long long* counts, int* term_table, double* coef);

/* The same export for the adjoint plan (pi_plan_adjoint). */
int pi_stencil_export_adjoint(int N, int d, int nsectors, const int* sector_ks, int nterms,
                              const int* term_kind, const double* ops, const double* rates,
                              const double* hbar, long long* counts, int* term_table,
                              double* coef);

/* Dense block of the collective operator sum_i X_i in sector (N-k, k), column-major
 * interleaved complex n x n (geometry.jl:1238-1256); op is 2x2 column-major interleaved. */
int pi_collective_block(int N, int k, const double* op, double* out);

/* f^(N-k,k) (partitions.jl:119-127) rounded to double, and its square root. */
int pi_sector_multiplicity(int N, int k, double* f, double* sqrt_f);

/* ---- apply!(y, compiled, x, t, p, work) (liouvillian.jl:4165-4171, :3205-3230) ------ */

/* y = L x for ncols right-hand sides with leading dimension ld (elements), device
 * buffers, complex FP64 reference coordinates, enqueued on `stream` (a cudaStream_t;
 * NULL is the CUDA default stream) without synchronizing.
 * Aliasing of x and y is rejected (liouvillian.jl:3220-3221). */
int pi_apply_f64(pi_plan* plan, double* y_dev, const double* x_dev, int ncols, long long ld,
                 void* stream);
/* Same action in complex FP32, in reference (x) or population (z = sqrt(f) x)
 * coordinates (PI_COORDS_*).  Population coordinates keep every sector inside the FP32
 * exponent range (stored PI coefficients of large-f sectors fall below 1e-38 near N=300). */
int pi_apply_f32(pi_plan* plan, float* y_dev, const float* x_dev, int ncols, long long ld,
                 int coords, void* stream);
/* Batched FP32 action on an element-major batch: y[e*ld + c] = (L x_c)[e] for the ncols
 * right-hand sides c (a (dim, ncols) row-major array of complex values, e.g. a batch of
 * Krylov vectors or initial states kept side by side).  Replaces the matrix form of
 * apply! (liouvillian.jl:3232-3251) for a batch held in this layout.  ncols and ld even,
 * both buffers 16-byte aligned.  Needs a plan whose stencil sits at the canonical
 * positions (pi_plan_info_t.batched_kernel == 2).  Kernels: TMA-staged tiles of 16, 32 or
 * (without pumping terms) 64 rows for plans of up to 160 sectors (N <= 318; tensor maps
 * encoded on the host per source pointer, stride and width, the last four kept), and plain
 * loads.  Autotuned: the first call for a batch width and coordinate system runs every
 * candidate on the caller's batch, times them with CUDA events on `stream`, waits for that
 * stream once and keeps the fastest for later calls; all candidates give the same y.  The
 * coefficient planes (32-48 bytes per PI coordinate for TMA, 80-112 for plain loads) are
 * built and cached on first use, with a synchronisation of their own.  A caller that
 * captures the apply into a CUDA graph therefore makes one call per batch width and
 * coordinate system before the capture. */
int pi_apply_f32_em(pi_plan* plan, float* y_dev, const float* x_dev, int ncols, long long ld,
                    int coords, void* stream);
/* The element-major kernel in use for (ncols, coords): kind 0 TMA-staged with tiles of
 * *rows rows, 1 plain loads; *ms = the autotuner's timed duration of one apply (0 when the
 * choice was pinned).  PI_ERR_INVALID_ARGUMENT before the first call with that width and
 * coordinate system.  No counterpart in the reference (its autotuner-free CPU path). */
int pi_apply_f32_em_tuning(pi_plan* plan, int ncols, int coords, int* kind, int* rows, double* ms);
/* Pins the element-major kernel for (ncols, coords) instead of autotuning it (kind and rows
 * as above; PI_ERR_INVALID_ARGUMENT for a choice the plan does not offer).  No counterpart
 * in the reference. */
int pi_apply_f32_em_select(pi_plan* plan, int ncols, int coords, int kind, int rows);
/* Convenience with host buffers: copies x in, applies, copies y out (pinned host memory
 * gives full link bandwidth).  The FP32 variant takes PI_COORDS_* like pi_apply_f32. */
int pi_apply_host_f64(pi_plan* plan, double* y_host, const double* x_host, int ncols);
int pi_apply_host_f32(pi_plan* plan, float* y_host, const float* x_host, int ncols, int coords);

/* ---- observables (highlevel.jl:665-677) --------------------------------------------- */

/* Device dot(a, b) = sum conj(a) b, FP64, deterministic two-stage reduction. */
int pi_dot_f64(pi_plan* plan, const double* a_dev, const double* b_dev, double* out_host2);

/* Allocation-free multi-dot: h_dev[i] = sum_e conj(V_i[e]) w[e] for i < nv, with V the nv
 * columns of length n at leading dimension ldv (complex FP64, device).  No counterpart in
 * the reference.  For callers that cannot call cudaMalloc when they need a reduction --
 * device memory owned by another pool (a Julia caller's CUDA.jl allocator), serving loops
 * that fix their memory at start-up, enqueueing while a stream is captured -- its partial
 * sums live in a static device array inside this library (128 KiB, kept on every GPU that
 * loads the library until exit), so it allocates nothing.  nv is limited to 32 (larger nv
 * is rejected).  Every call looks up the array's device address on the current device (a
 * host-side lookup, valid again after a device reset); a CUDA error left pending by earlier
 * work is reported, not cleared.  Calls share the array: two calls that overlap on the GPU
 * race.  Asynchronous on `stream` (NULL = default stream).  The harmonic and implicitly
 * restarted Arnoldi drivers (krylov.jl:996-1110, 1378-1551) project through it, in groups of
 * at most 32 basis vectors. */
int pi_mdot_f64_noalloc(const double* V_dev, long long ldv, int nv, const double* w_dev, long long n,
                        double* h_dev, void* stream);

/* ---- Arnoldi factorisation for Liouvillian spectra (krylov.jl:914-962) -------------
 * krylov_liouvillian_spectrum's Krylov process on the device: V[:,0] = v0/|v0|, then for
 * j = 0..m-1: w = L V[:,j]; two Gram-Schmidt passes against V[:,0..j] (their sum is column
 * j of H); H[j+1,j] = |w|; stop after step m or when H[j+1,j] <= eps * |L V[:,j]| (the
 * reference's breakdown test); else V[:,j+1] = w / H[j+1,j].  The k x k Hessenberg
 * eigenproblem, Ritz ordering and residual estimates stay with the caller, as the
 * reference hands them to its LAPACK (_projected_eigen, krylov.jl:31-40).  FP64. */
typedef struct {
  int steps;          /* k: Arnoldi steps taken (columns of H filled) */
  int breakdown;      /* 1 when the breakdown test stopped the process before step m */
  int operator_applications;
} pi_arnoldi_info_t;

/* v0_dev: dim complex (not modified); V_dev: (m+1) columns of dim complex at leading
 * dimension ldv >= dim, written; H_host: (m+1) x m complex column-major, zero-filled
 * then written.  1 <= m <= 127. */
int pi_arnoldi(pi_plan* plan, const double* v0_dev, int m, double* V_dev, long long ldv,
               double* H_host, pi_arnoldi_info_t* info);

/* out[:, c] = sum_i coef[i + c*k] V[:, i] for c < ncols: Ritz vectors from an Arnoldi basis
 * (V: k columns of dim complex at ldv; coef: k x ncols complex column-major on the host;
 * out: ncols columns at ldo, device).  FP64. */
int pi_combine_f64(pi_plan* plan, const double* V_dev, long long ldv, int k, const double* coef_host,
                   int ncols, double* out_dev, long long ldo);

/* ---- steady state: krylov_steady_state (krylov.jl:797-891) -------------------------- */

/* Level-sweep preconditioner: replaces schur_sector_preconditioner (krylov.jl:594-700),
 * which LU-factors the dense n^2 x n^2 Schur blocks of L/s + v t^H (O(n^6) per sector).
 * This one inverts, exactly and in O(dim) work, M = L0/s + v t^H, where L0 keeps every term
 * of L that preserves the charge m - m' (all Jz-covariant dissipators, the diagonal of the
 * Hamiltonian) and drops the terms that change it (a Jx or Jy drive).  L0 is block diagonal
 * in the charge and, inside a charge block, block triangular over the levels m with
 * tridiagonal blocks over the sectors, so one thread block per charge sweeps the levels
 * with precomputed Thomas factors.  Used on the left in GMRES exactly like the reference's
 * preconditioner argument (_gmres!, krylov.jl:732-787).  Models whose charge-keeping gains
 * both raise and lower m (decay and pumping together) are rejected with
 * PI_ERR_UNSUPPORTED; a singular level block without the single free dark-state entry
 * needs regularization > 0 (added to the diagonal of L0/s, as in the reference).
 * coords: PI_COORDS_POPULATION (FP32 sweeps; the coordinates whose norms weigh
 * populations, the ones to use at large N) or PI_COORDS_REFERENCE (FP64 sweeps).
 * operator_scale: 0 = estimate from 3 random probes in those coordinates.  The tables take
 * about 64 bytes (population) or 120 bytes (reference) per PI coordinate. */
typedef struct pi_precond pi_precond;
typedef struct {
  int coords;
  int fp64;               /* sweep arithmetic: 1 FP64, 0 FP32 */
  double operator_scale;  /* s */
  double regularization;
  int chains;             /* charge chains (thread blocks per apply) */
  int levels;             /* (charge, level) blocks */
  long long entries;      /* = dim */
  int max_level;          /* sectors in the largest level block */
  int direction;          /* -1: levels swept from high m to low m (decay-type gains) */
  int singular;           /* 1: L0 singular, its free entry fixed by the trace */
  size_t device_bytes;
  double setup_seconds;
  int kind;                 /* PI_PRECOND_LEVEL or PI_PRECOND_DRIVE */
  double max_asymmetry;     /* drive: largest |H_ab - H_ba| of the sector Hamiltonian blocks */
  double max_nonhermitian;  /* drive: largest real row-shift coefficient left out */
} pi_precond_info_t;
enum { PI_PRECOND_LEVEL = 0, PI_PRECOND_DRIVE = 1 };
int pi_precond_create(pi_plan* plan, int coords, double regularization, double operator_scale,
                      pi_precond** out);
/* Drive preconditioner (PI_PRECOND_DRIVE): per Schur sector the commutator with H_s (the
 * sector's Hamiltonian block, real symmetric tridiagonal) and the diagonal, in H_s's
 * orthogonal eigenbasis, of the loss anticommutator, solved exactly there
 * (X = U [(U^T R U) ./ d] U^T, d_ij = (-i (h_i - h_j) - (q_i + q_j) / 2) / s, q_i the loss
 * eigenmode i sees, floored at half the sector's mean loss), with the trace border v t^H by
 * Sherman-Morrison; FP64 vectors in FP64 arithmetic (the plain FP64 solve), FP32 vectors in
 * FP32 (the mixed solve's inner steps).  It carries the drive exactly and leaves out the loss
 * coupling between eigenmodes, the sandwich gains and the coupling between sectors, which
 * the level sweep (pi_precond_create) carries exactly where the drive does not dominate.  As opts.preconditioner GMRES applies it twice per
 * step (z = D r; z += D (r - B z), B the bordered operator).  The host eigendecompositions run
 * on the host threads.  The reference's preconditioner for the same system is the dense LU of
 * every sector block of L/s + v t^H (krylov.jl:594-699), infeasible beyond N ~ 40. */
int pi_precond_create_drive(pi_plan* plan, int coords, double operator_scale, pi_precond** out);
int pi_precond_destroy(pi_precond* precond);
int pi_precond_info(const pi_precond* precond, pi_precond_info_t* out);
/* z = M^-1 r (complex FP64 device vectors in the preconditioner's coordinates), enqueued on
 * `stream`; the ldiv! of the reference's preconditioner object (krylov.jl:202-209). */
int pi_precond_apply(const pi_precond* precond, double* z_dev, const double* r_dev, void* stream);

/* Host-only inspection (no device): the tables pi_precond_create would upload for the model
 * of pi_stencil_export's arguments, in FP64 (the sweep kernel reads them in FP32 for
 * population coordinates).  Entries are ordered by charge chain, level (in sweep order) and
 * sector.  Two-call pattern: with tables NULL only counts[0..3] = chains, levels, entries and
 * d = 0 chain entries are written.  No counterpart in the reference. */
typedef struct {
  int* chain_lev;      /* chains + 1: first level record of every chain */
  int* lev_ent;        /* levels + 1: first entry of every level record */
  int* elem;           /* entries: element index in the PI vector */
  double* W;           /* entries complex: 1/pivot (forward y_i = W_i r_i + A_i y_{i-1}) */
  double* A;           /* entries complex */
  double* C;           /* entries complex (backward u_i = y_i + C_i u_{i+1}) */
  int* gsrc;           /* entries: three 10-bit sector positions in the previous level (1023 none) */
  double* G;           /* 3 x entries complex: the gain coefficients */
  double* t0;          /* d = 0 chain entries: trace weights */
  double* v0;          /* d = 0 chain entries: the border vector v */
  double* w0;          /* d = 0 chain entries complex: the sweep y_v of s v with the free equation
                          dropped (mode 0) or s L0^-1 v (mode 1) */
  int meta[8];         /* chain0, chain0_ent, mode (0 free entry, 1 Sherman-Morrison), free_ent,
                          direction, max_level */
  double sm_coef[2];   /* rho_v, the dropped equation's residual for s v (mode 0), or
                          1 / (1 + t^H w0) (mode 1) */
} pi_precond_tables_t;
int pi_precond_export(int N, int d, int nsectors, const int* sector_ks, int nterms, const int* term_kind,
                      const double* ops, const double* rates, const double* hbar, int coords,
                      double regularization, double operator_scale, long long* counts,
                      pi_precond_tables_t* tables);
/* Host-only inspection of the drive preconditioner's tables for the same model arguments:
 * counts[0..2] = sectors, sum n_s^2, sum n_s; with U, h, c, q non-NULL also the eigenvector
 * pool (sector by sector, n_s x n_s column-major, column i the eigenvector of h[i]), the
 * eigenvalue pool, c_s = -2 x the mean loss of every sector and, per eigenmode, the loss it
 * sees (U^T Q U)_ii floored at -c_s / 4 (all unscaled). */
int pi_precond_drive_export(int N, int d, int nsectors, const int* sector_ks, int nterms, const int* term_kind,
                            const double* ops, const double* rates, const double* hbar, long long* counts,
                            double* U, double* h, double* c, double* q);

typedef struct {
  int krylovdim;          /* GMRES restart length m (default 30) */
  int maxiter;            /* total Arnoldi steps (default 500) */
  double atol, rtol;      /* defaults 1e-10, 1e-8 */
  double operator_scale;  /* <= 0: estimate from 3 random probes (krylov.jl:156-169) */
  int precision;          /* PI_FP64, or PI_FP32 = FP32 inner applies with FP64 refinement */
  int use_initial;        /* 1: x_dev holds the initial state; 0: start from v = t/|t|^2 */
  int max_refinements;    /* PI_FP32 only: outer FP64 refinement cycles (default 200) */
  int coords;             /* coordinates of the solve (PI_COORDS_*, default reference): in
                             population coordinates the residual and trace tests weigh
                             populations (the reference-coordinate norms of high-multiplicity
                             sectors vanish at large N); x_dev stays in reference coordinates */
  const pi_precond* preconditioner;  /* NULL (default) or a left preconditioner built for the
                             same plan and coordinates; its operator scale is used */
  const pi_precond* drive_preconditioner;  /* NULL (default), or with a PI_PRECOND_LEVEL
                             `preconditioner` a PI_PRECOND_DRIVE one of the same plan, coordinates
                             and scale: the solve starts with the level sweep and moves, after a
                             restart cycle that reduced the raw residual by less than 3x, to the
                             drive part applied twice, and after a cycle of that stage that
                             gained less than 1.25x to drive, level and drive in turn
                             (regime-adaptive; no reference counterpart) */
} pi_gmres_opts_t;

typedef struct {
  int converged;
  int iterations;           /* Arnoldi steps */
  int restarts;
  int refinements;          /* PI_FP32 outer cycles */
  int operator_applications;
  double residual;          /* ||L x|| */
  double normalized_residual; /* ||L x|| / s */
  double trace_error;       /* |t^H x - 1| */
  double operator_scale;
  double linear_residual;
  int preconditioner_stage; /* with both preconditioners: 0 level, 1 drive x2, 2 drive-level-drive */
} pi_gmres_info_t;

void pi_gmres_default_opts(pi_gmres_opts_t* opts);
/* Solves for the trace-one stationary state into x_dev (complex FP64, device, reference
 * coordinates).  The info residuals are those of the solve's coordinates.  With a
 * preconditioner the convergence tests are the reference's preconditioned ones: the
 * preconditioned residual against atol + rtol |P b| and the raw residual against
 * atol + rtol |b| (krylov.jl:739-786). */
int pi_steady_state(pi_plan* plan, double* x_dev, const pi_gmres_opts_t* opts,
                    pi_gmres_info_t* info);

/* ---- time evolution: krylov_expv! (krylov_extensions.jl:1452-1573) ------------------- */

typedef struct {
  int krylovdim;         /* default 30 */
  double atol, rtol;     /* defaults 1e-10, 1e-8 */
  double initial_step;   /* <= 0: nothing */
  double minimum_step;   /* <= 0: nothing */
  double maximum_step;   /* <= 0: nothing */
  int max_steps;         /* default 10000 */
  double safety;         /* default 0.9 */
  int precision;         /* PI_FP64, or PI_FP32 = FP32 applies with FP64 orthogonalisation */
} pi_expv_opts_t;

typedef struct {
  int converged;
  double reached_time;
  int accepted_steps, rejected_steps;
  int operator_applications;
  int arnoldi_factorizations;
  int trial_evaluations;
  double estimated_error;
} pi_expv_info_t;

void pi_expv_default_opts(pi_expv_opts_t* opts);
/* x_dev <- exp(t L) x_dev (complex FP64, device). */
int pi_expv(pi_plan* plan, double* x_dev, double t, const pi_expv_opts_t* opts,
            pi_expv_info_t* info);

/* solve_dynamics(..., algorithm=ExpvAlgorithm(...), saveat=times, observables=obs,
 * save_states=false) (highlevel.jl:559-733): propagates rho (device, in place) through
 * the nt saved times and writes nobs complex expectation values per time into
 * values_host[(it*nobs + o)*2 + {0,1}]; obs_dev holds nobs observable vectors of
 * length dim (PIOperator data) back to back. */
int pi_solve_dynamics(pi_plan* plan, double* rho_dev, int nt, const double* times,
                      int nobs, const double* obs_dev, double* values_host,
                      const pi_expv_opts_t* opts, pi_expv_info_t* info);

/* ---- fixed-step RK4 (the reference's default dynamics algorithm) ---------------------
 * evolve! (evolution.jl:75-118): steps classical RK4 steps of h = (t1 - t0) / steps with
 * the reference's stage sequence and three scratch vectors.  Each step is four fused
 * launches: the stencil apply of one stage with that stage's vector updates as its
 * epilogue; the steps of one saved interval run as one CUDA graph.  PI_FP32 applies the
 * operator in FP32 population coordinates (z = sqrt(f) x) while the state and the stage
 * sum stay FP64. */
typedef struct {
  int steps_per_interval;  /* > 0; solve_dynamics' default is 64, evolve!'s is 256 */
  int precision;           /* PI_FP64 or PI_FP32 */
} pi_rk4_opts_t;

typedef struct {
  long long steps;                  /* RK4 steps taken */
  long long operator_applications;  /* 4 per step */
  double reached_time;
} pi_rk4_info_t;

void pi_rk4_default_opts(pi_rk4_opts_t* opts);

/* evolve!(dest, L, src, (t0, t1); steps): dest_dev <- RK4 propagation of src_dev (device,
 * complex FP64).  dest may equal src; partially overlapping storage is rejected
 * (evolution.jl:83-84); steps must be positive (:82). */
int pi_evolve(pi_plan* plan, double* dest_dev, const double* src_dev, double t0, double t1,
              const pi_rk4_opts_t* opts, pi_rk4_info_t* info);

/* solve_dynamics(..., algorithm=:auto | :rk4, saveat=times, steps_per_interval,
 * observables=obs, save_states=false) (highlevel.jl:559-566, 693-733): RK4 over every
 * saved interval, zero-length intervals skipped; the layout of times, obs_dev and
 * values_host is pi_solve_dynamics's. */
int pi_solve_dynamics_rk4(pi_plan* plan, double* rho_dev, int nt, const double* times,
                          int nobs, const double* obs_dev, double* values_host,
                          const pi_rk4_opts_t* opts, pi_rk4_info_t* info);

/* ---- batched solves over many plans (parameter scans, mixed particle numbers) --------
 * One engine advances every instance together: each Arnoldi step of all instances is one
 * launch per kernel over an (instance, sector-tile) or (instance, element-chunk) work list,
 * each Krylov cycle runs as one CUDA graph with the step index and stop flags in device
 * memory, and the host runs the reference's controller per instance between cycles.  An
 * instance's arithmetic does not depend on the other instances in the batch.  The plans
 * are only read (several instances may share one plan); state buffers must be distinct.
 * The reference has no batched entry point: these replace a loop over parameter points
 * that calls solve_dynamics / stationary_state (scans.jl:1457 parameter_scan) per point.
 * krylovdim is limited to 1..120.  Returns PI_OK when every instance succeeded, else the
 * first failing instance's status (its message names the instance); infos[i] is filled
 * for every instance either way. */

/* Batched krylov_expv!: x_devs[i] <- exp(t[i] L_i) x_devs[i]. */
int pi_expv_batch(int ninst, pi_plan* const* plans, double* const* x_devs, const double* t,
                  const pi_expv_opts_t* opts, pi_expv_info_t* infos);

/* One job of pi_dynamics_batch: pi_solve_dynamics's arguments for one instance. */
typedef struct {
  pi_plan* plan;
  double* state_dev;      /* in: initial state, out: state at times[nt-1] (device) */
  int nt;                 /* saved times (>= 1), nondecreasing */
  const double* times;    /* host */
  int nobs;               /* 0..16 observables */
  const double* obs_dev;  /* nobs x dim complex (device) */
  double* values_host;    /* nt x nobs complex: values[(it*nobs + o)*2 + {0,1}] */
} pi_dynamics_job_t;

/* Batched solve_dynamics(...; algorithm=ExpvAlgorithm, saveat, observables,
 * save_states=false) (highlevel.jl:559-733). */
int pi_dynamics_batch(int njobs, const pi_dynamics_job_t* jobs, const pi_expv_opts_t* opts,
                      pi_expv_info_t* infos);

/* Batched stationary states (krylov.jl:797-891) into x_devs[i].  The operator-scale
 * probes come from a counter-based generator on the device (seeded per call), so the
 * estimated scale agrees with pi_steady_state's to tolerance, not bitwise. */
int pi_steady_state_batch(int ninst, pi_plan* const* plans, double* const* x_devs,
                          const pi_gmres_opts_t* opts, pi_gmres_info_t* infos);

/* Schedule of the FP32 Arnoldi-step apply of the batched engine (the batched entry points
 * above and PI_FP32 servers).  PI_SCHEDULE_PER_TILE launches one block per (instance,
 * sector-tile) item; k >= 1 launches k blocks per SM (clamped to the resident limit) that
 * walk the item list persistently, prefetching each next tile's staged windows while
 * computing the current one.  PI_SCHEDULE_AUTO (the default) times every candidate with
 * CUDA events on the engine stream before the first Krylov cycle of a job set whose shape
 * (work-list size class, canonical or general stencils) has not been seen by that engine,
 * and keeps the fastest; the timed launches write only the step's scratch column, which
 * the cycle recomputes.  Every schedule gives bitwise the same results.  Process-wide;
 * applies to engines that choose a schedule after the call. */
enum { PI_SCHEDULE_AUTO = 0, PI_SCHEDULE_PER_TILE = -1 };
int pi_engine_set_apply_schedule(int schedule);

typedef struct {
  int choices;        /* schedules chosen so far, process-wide (tuned or cached or set) */
  int tunings;        /* of which timed */
  int schedule;       /* the last choice: PI_SCHEDULE_PER_TILE or blocks per SM */
  int items;          /* work-list items of the job set it was made for */
  int resident_max;   /* resident blocks per SM of the persistent launch */
  int ncand;          /* candidates of the last timing (0 if the last choice was not timed) */
  int cand[8];        /* PI_SCHEDULE_PER_TILE or blocks per SM */
  double cand_us[8];  /* median launch time of each, microseconds */
} pi_schedule_info_t;
int pi_engine_schedule_info(pi_schedule_info_t* out);

/* ---- serving: continuous batching of time-evolution and steady-state requests --------
 * A server owns one batched engine and a worker thread.  Requests are admitted in arrival
 * order between engine ticks while their device footprint (Krylov basis, image and state
 * vectors; the plan tables belong to the caller) fits memory_budget and fewer than
 * max_active requests run; admitted requests join the next tick's batched launches and
 * keep their states and Krylov bases resident until they finish.  A request's arithmetic
 * does not depend on the other requests it shares ticks with.  The reference has no
 * serving layer; a request is the work of one solve_dynamics(...; saveat=dt) call
 * (highlevel.jl:559-733) or one stationary_state call (krylov.jl:797-891).
 * The caller keeps the plan, the state buffer and any observable buffers alive and
 * untouched until the request's completion has been polled; the state is complete when
 * the completion is posted. */
typedef struct pi_server pi_server;

typedef struct {
  int krylovdim;         /* Krylov dimension of every request (default 30, <= 120) */
  int precision;         /* PI_FP64, or PI_FP32 (FP32 applies and basis, FP64 rest) */
  double memory_budget;  /* device bytes admitted requests may hold (default 160e9) */
  int max_active;        /* concurrent requests, 0 = unlimited */
  int use_graphs;        /* capture each Krylov cycle as a CUDA graph (default 1) */
  int steady_solvers;    /* 0 (default): steady-state requests run unpreconditioned in the
                            batched engine (the reference's method).  k > 0: k host threads solve
                            them beside the engine, each request with its own level and drive
                            preconditioners (population coordinates, the adaptive ladder of
                            pi_gmres_opts_t.drive_preconditioner; unpreconditioned, the
                            reference's method, where the level sweep does not apply),
                            GMRES(max(krylovdim, 50)) in the server's precision on the plan's
                            stream; maxiter defaults to 2000 */
} pi_server_opts_t;

enum { PI_REQUEST_DYNAMICS = 0, PI_REQUEST_STEADY = 1 };

typedef struct {
  int kind;                  /* PI_REQUEST_DYNAMICS or PI_REQUEST_STEADY */
  pi_plan* plan;
  double* state_dev;         /* dynamics: initial state in, final state out; steady: output */
  double t_final;            /* dynamics: saved times 0:dt:t_final (+ t_final) */
  double dt;
  double atol, rtol;         /* <= 0: the solver defaults (1e-10, 1e-8) */
  int maxiter;               /* steady: <= 0 default 500 */
  int nobs;                  /* dynamics: 0..16 observables, values at every saved time */
  const double* obs_dev;
  double* values_host;       /* nt x nobs complex (nt from the saved-time grid) */
  unsigned long long tag;    /* caller's request id, returned in the completion */
} pi_request_t;

typedef struct {
  unsigned long long tag;
  int kind;
  int status;                /* PI_OK or the request's error code */
  double submit_time;        /* seconds since pi_server_create */
  double start_time;         /* admission */
  double finish_time;
  int iterations;            /* dynamics: accepted steps; steady: GMRES iterations */
  int operator_applications;
  double residual;           /* dynamics: summed error estimate; steady: normalized residual */
  double trace_error;        /* steady */
  char message[160];
} pi_completion_t;

typedef struct {
  long long submitted, admitted, completed, queued, active;
  double bytes_in_use;
  long long ticks, cycles, arnoldi_steps;
  double elapsed;
} pi_server_stats_t;

void pi_server_default_opts(pi_server_opts_t* opts);
int pi_server_create(const pi_server_opts_t* opts, int device, pi_server** out);
/* Thread-safe, non-blocking.  PI_ERR_OUT_OF_MEMORY when the request alone exceeds the budget. */
int pi_server_submit(pi_server* server, const pi_request_t* request);
/* Returns up to max completions; waits up to timeout_ms (< 0: until one is available). */
int pi_server_poll(pi_server* server, pi_completion_t* out, int max, int* count, int timeout_ms);
int pi_server_stats(pi_server* server, pi_server_stats_t* stats);
/* Stops after the current tick; unfinished requests are abandoned. */
int pi_server_destroy(pi_server* server);

#ifdef __cplusplus
}
#endif

#endif /* PICUDA_H */
