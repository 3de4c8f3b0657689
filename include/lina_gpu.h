/*
 * lina_gpu.h - the thin C-ABI between LinA host code and the GB300 (sm_103a)
 * kernels of the sparse solve path.
 *
 * Plain pointers and sizes only.  Matrices are CSR with int32 row pointers
 * and column indices (columns sorted within a row, explicit zeros allowed) and
 * FP64 values, which is the reference's row-list sparse_matrix
 * (LinA/linear_algebra.h:29-34) laid out contiguously.  One process, one GPU,
 * one host thread: like the reference (whose solver state lives in
 * file-static globals), the library is not thread-safe.
 *
 * Return codes: 0 on success, a negative LINA_GPU_E* code on failure; the
 * text of the last failure is available from lina_gpu_last_error().
 */
#ifndef LINA_GPU_H
#define LINA_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LINA_GPU_OK 0
#define LINA_GPU_EINVAL -1      /* invalid argument                            */
#define LINA_GPU_ECUDA -2       /* CUDA runtime error (allocation, launch)     */
#define LINA_GPU_ESETUP -3      /* AMG setup hit a condition the reference aborts on */
#define LINA_GPU_EBREAKDOWN -4  /* Krylov breakdown (zero or NaN inner product) */
#define LINA_GPU_ENOCONV -5     /* iteration limit reached before the tolerance */

/* coarsening strategies, values of LinA/Multigrid.h:29-31, and PMIS: an opt-in extension that
   computes the C/F labels on the GPU as a parallel independent set (fast set-up; labels, and so
   hierarchies and iteration counts, differ from the reference's sequential coarsening) */
#define LINA_AGGRESSIVE 1
#define LINA_STANDARD 2
#define LINA_PMIS 3

/* smoothers of the GPU V-cycle */
#define LINA_SMOOTHER_JACOBI 0   /* damped Jacobi, x += w D^-1 (b - A x)                 */
#define LINA_SMOOTHER_MC_SOR 1   /* SOR over a greedy multicolouring, colours in order    */

/* precision of the preconditioner */
#define LINA_PREC_FP64 0         /* everything FP64                                      */
#define LINA_PREC_MIXED 1        /* FP32 V-cycle (values, vectors, accumulation), FP64 coarse solve,
                                    FP64 flexible CG outside                              */

/* stopping rules of lina_gpu_pcg */
#define LINA_STOP_REFERENCE 0    /* ||r_k|| / ||M^-1 r_0|| <= tol, as pcg (LinA/PCGS.c:191-213) */
#define LINA_STOP_RELATIVE 1     /* ||r_k|| / ||b|| <= tol, confirmed on the true residual b - A x */

/* flags of lina_gpu_pcg */
#define LINA_PCG_DEVICE_PTRS 1   /* b and x are device pointers (default: host pointers)  */
#define LINA_PCG_USE_X0 2        /* start from the given x (default: x = 0)               */
#define LINA_PCG_FINAL_PRECON 4  /* apply M^-1 once more after the loop for the reference's
                                    pcg residuum (LinA/PCGS.c:217-218)                    */
#define LINA_PCG_TIME_KERNELS 8  /* time the smoother sweeps of the level with the most stored entries
                                    (the dominant kernel) with CUDA events                 */
#define LINA_PCG_NORMALIZE 16    /* scale b and x by 1/||b|| during the solve, as pcg does */
#define LINA_PCG_HOST_LOOP 32    /* drive every iteration from the host instead of the captured
                                    CUDA graph with its device-side while loop              */
#define LINA_PCG_BETA_FLEXIBLE 256  /* beta = -alpha_prev (z.q_prev) / s_old (flexible CG), the default
                                       for LINA_PREC_MIXED                                   */
#define LINA_PCG_BETA_STANDARD 512  /* beta = s / s_old (the reference's, LinA/PCGS.c:200), the default
                                       for LINA_PREC_FP64                                    */

typedef struct lina_gpu_amg lina_gpu_amg;

typedef struct lina_gpu_amg_options {
    int dof;                       /* unknowns per node, block ordering [u0 ..., u1 ...]  */
    int depth;                     /* number of levels                                    */
    int smoothing_iterations;      /* sweeps per pre/post smoothing                       */
    int aggr_smoothing_iterations; /* sweeps on the finest level when coarsening is aggressive */
    int coarsening;                /* LINA_AGGRESSIVE, LINA_STANDARD or LINA_PMIS         */
    double eps_minus, eps_plus;    /* strength thresholds (set_connection_thresholds)     */
    double matrix_tol;             /* interpolation truncation (AMG_set_matrix_tolerance) */
    int smoother;                  /* LINA_SMOOTHER_*                                     */
    double omega;                  /* relaxation factor of the smoother                   */
    int precision;                 /* LINA_PREC_*                                         */
} lina_gpu_amg_options;

typedef struct lina_gpu_solve_info {
    int iterations;
    int status;                    /* 0 or a negative LINA_GPU_E* code                    */
    double rel_residual;           /* value tested by the stopping rule at exit           */
    double true_rel_residual;      /* ||b - A x|| / ||b|| recomputed in FP64 at exit       */
    double pcg_residuum;           /* ||M^-1 r|| / ||M^-1 r_0|| (LINA_PCG_FINAL_PRECON)    */
    double smoother_ms;            /* total time of the timed smoother launches           */
    int smoother_launches;         /* number of timed smoother launches                   */
    double smoother_bytes;         /* algorithmic bytes of one timed launch               */
    int timed_level;               /* level of the timed sweeps: the one with most entries */
    int timed_rows;                /* its rows                                            */
    long timed_entries;            /* its stored entries                                  */
    int restarts;                  /* restarts of the recurrence from the true residual   */
} lina_gpu_solve_info;

void lina_gpu_default_options(lina_gpu_amg_options* opt);

/* AMG_setup (LinA/Multigrid.c:1613) on a CSR matrix: host setup, then upload of every level. */
int lina_gpu_amg_create(int n, const int* rowptr, const int* col, const double* val,
                        const lina_gpu_amg_options* opt, lina_gpu_amg** out);
/* the same setup without touching the GPU (hierarchy inspection and tests on machines without one);
   the handle supports only the inspection functions below and lina_gpu_amg_destroy */
int lina_gpu_amg_create_host_only(int n, const int* rowptr, const int* col, const double* val,
                                  const lina_gpu_amg_options* opt, lina_gpu_amg** out);
/* AMG_recompute_coarse_matrices (LinA/Multigrid.c:1756): new fine matrix, same P and R. */
int lina_gpu_amg_recompute(lina_gpu_amg* h, int n, const int* rowptr, const int* col, const double* val);
/* New values for the finest matrix on the pattern given at creation (val[nnz], host pointer, or
   device pointer with LINA_PCG_DEVICE_PTRS).  The Krylov operator, the finest smoother and its
   diagonal take the new values; coarse levels keep the setup's (a preconditioner built for a
   nearby matrix), so no host work is done.  No reference counterpart: AMG_recompute_coarse_matrices
   (lina_gpu_amg_recompute) is the exact re-setup.  EINVAL for one-level hierarchies and for
   matrices whose rows were sign-flipped at setup. */
int lina_gpu_amg_update_values(lina_gpu_amg* h, const double* val, int flags);
int lina_gpu_amg_destroy(lina_gpu_amg* h);
/* Save a hierarchy to the directory dir (created if missing): every level's A, P and R in the
   reference's write_sparse format (LinA/linear_algebra.c:832), labels and unknown numbers as int
   arrays, the setup parameters in hierarchy.txt.  No reference counterpart: it lets a later run skip
   AMG_setup. */
int lina_gpu_amg_save(const lina_gpu_amg* h, const char* dir);
/* A hierarchy saved by lina_gpu_amg_save, uploaded (or host-only when host_only is nonzero).  The
   structure (depth, dof, coarsening, thresholds) comes from the files, the solve options (smoother,
   omega, precision, sweeps) from opt; the coarsest factorisation is recomputed.  The result solves
   exactly as the saved hierarchy did. */
int lina_gpu_amg_load(const char* dir, const lina_gpu_amg_options* opt, int host_only, lina_gpu_amg** out);
/* change smoother, relaxation or precision of an existing hierarchy */
int lina_gpu_amg_set_smoother(lina_gpu_amg* h, int smoother, double omega, int precision);
/* Krylov directions kept by lina_gpu_pcg and the batch solves (no reference counterpart): m >= 2 runs the
   truncated flexible CG FCG(m) of Notay, which makes every new direction A-orthogonal to the last m
   (robust to the slight variation of the FP32 V-cycle between applications); m = 1 the two-term
   recurrences (flexible beta in mixed precision, the reference's beta in FP64); 0 (default) FCG(6) in mixed
   precision and the reference's CG in FP64.  Up to 8.  The LINA_PCG_BETA_* flags select the two-term
   recurrence for one call.  FCG(m) keeps 2 m extra FP64 vectors on the device. */
int lina_gpu_amg_set_fcg_history(lina_gpu_amg* h, int m);

/* AMG-preconditioned CG on the hierarchy's finest matrix (pcg, LinA/PCGS.c:163). */
int lina_gpu_pcg(lina_gpu_amg* h, const double* b, double* x, double tol, int max_iter,
                 int stop_rule, int flags, lina_gpu_solve_info* info);
/* Batched AMG-PCG over independent systems (no reference counterpart: the reference solves them
   one pcg call at a time).  One CUDA graph holds a branch per system: x = 0, the PCG loop of
   lina_gpu_pcg on the device and the true residual.  One launch solves all systems concurrently.
   The hierarchies stay owned by the caller.  They must outlive the batch, keep the smoother and
   precision they had at creation, and be used by nothing else while a batch solve runs.  A system
   may appear once.  stop_rule as for lina_gpu_pcg.  With LINA_STOP_RELATIVE, a system whose true
   residual misses tol continues from the batch's x on its own (lina_gpu_pcg restarts from the
   true residual); infos[i] then counts both parts. */
typedef struct lina_gpu_batch lina_gpu_batch;
int lina_gpu_batch_create(int count, lina_gpu_amg* const* systems, int stop_rule, lina_gpu_batch** out);
/* b[i], x[i]: host arrays (device arrays with LINA_PCG_DEVICE_PTRS) of system i's size; infos may
   be NULL.  Returns 0, LINA_GPU_ENOCONV when a system did not converge, or another error. */
int lina_gpu_batch_solve(lina_gpu_batch* batch, const double* const* b, double* const* x, double tol,
                         int max_iter, int flags, lina_gpu_solve_info* infos);
int lina_gpu_batch_size(const lina_gpu_batch* batch);
int lina_gpu_batch_destroy(lina_gpu_batch* batch);
/* Segmented batch: the same independent systems solved as one.  Every level of one combined hierarchy
   is the block-diagonal concatenation of the systems' levels (a shallower system padded below its
   coarsest level with copies of it), the coarsest level is solved with each system's own dense
   inverse, and the Krylov loop is FCG(m) per system with segmented reductions (each system its own
   scalars and stopping test, ||b_i - A_i x_i|| <= tol ||b_i||, confirmed on the true residual with
   restarts): each kernel streams all systems' rows in one launch, and one graph launch runs until every
   system has stopped.  The systems must be device hierarchies with one smoother, precision and sweep
   count and no sign-flipped rows; the batch copies them at creation (later changes to a system do not
   reach it).  Solutions start from zero. */
typedef struct lina_gpu_segbatch lina_gpu_segbatch;
int lina_gpu_segbatch_create(int count, lina_gpu_amg* const* systems, lina_gpu_segbatch** out);
/* b[i], x[i] as for lina_gpu_batch_solve; infos may be NULL; flags: LINA_PCG_DEVICE_PTRS, and
   LINA_PCG_HOST_LOOP to launch the iterations from the host instead of the graph.  Returns 0,
   LINA_GPU_ENOCONV when a system did not converge, or another error. */
int lina_gpu_segbatch_solve(lina_gpu_segbatch* batch, const double* const* b, double* const* x, double tol,
                            int max_iter, int flags, lina_gpu_solve_info* infos);
/* the combined hierarchy: depth, and per level (0 = coarsest) rows and stored entries (arrays of depth) */
int lina_gpu_segbatch_levels(const lina_gpu_segbatch* batch, int* depth, long* rows, long* entries);
/* the combined hierarchy itself (owned by the batch; valid until lina_gpu_segbatch_destroy): a hierarchy
   of the block-diagonal system, usable with lina_gpu_pcg (one global recurrence over all systems), for
   example to time its kernels */
int lina_gpu_segbatch_hierarchy(lina_gpu_segbatch* batch, lina_gpu_amg** out);
int lina_gpu_segbatch_destroy(lina_gpu_segbatch* batch);
/* AMG_solve (LinA/Multigrid.c:1863): V-cycles from the initial guess X until ||F - A X|| / ||F - A X0||
   <= eps or max_iter cycles; flags may hold LINA_PCG_DEVICE_PTRS.  Returns the cycles done and the
   final relative residual. */
int lina_gpu_amg_solve(lina_gpu_amg* h, const double* F, double* X, double eps, int max_iter, int flags,
                       int* iterations, double* rel_residual);
/* AMG_solve with the FULL_AMG cycle structure (AMG_full_multigrid, LinA/Multigrid.c:1595): the
   right-hand side restricted to all levels, the coarsest solved, then on each finer level the
   prolongated solution improved by one V-cycle started from it.  X receives the result (its input
   is not used); *rel_residual = ||F - A X|| / ||F - A X_in||.  flags: LINA_PCG_DEVICE_PTRS. */
int lina_gpu_amg_fmg(lina_gpu_amg* h, const double* F, double* X, int flags, double* rel_residual);
/* one preconditioner application z = M^-1 r (device pointers), zero initial guess */
int lina_gpu_vcycle(lina_gpu_amg* h, const double* r_dev, double* z_dev);
/* y = A_level x on the device (level = depth-1 is the finest) */
int lina_gpu_spmv(lina_gpu_amg* h, int level, const double* x_dev, double* y_dev);

/* A single matrix on the device (the SpMV and smoother kernels without a hierarchy).
   Vectors are device pointers of FP64 (LINA_PREC_FP64) or FP32 (LINA_PREC_MIXED) elements. */
typedef struct lina_gpu_matrix lina_gpu_matrix;
int lina_gpu_matrix_create(int n, int ncols, const int* rowptr, const int* col, const double* val,
                           lina_gpu_matrix** out);
int lina_gpu_matrix_destroy(lina_gpu_matrix* m);
/* new values on the pattern given at creation (val[nnz] in CSR order; host pointer, or device
   pointer with LINA_PCG_DEVICE_PTRS): both value copies and the inverse diagonal are rewritten on
   the device, the layout is kept */
int lina_gpu_matrix_update_values(lina_gpu_matrix* m, const double* val, int flags);
/* y = A x */
int lina_gpu_matrix_spmv(lina_gpu_matrix* m, int precision, const void* x_dev, void* y_dev);
/* `sweeps` damped Jacobi sweeps x <- x + w D^-1 (b - A x); tmp is a work vector; after an odd
   number of sweeps the result is in tmp, after an even number in x */
int lina_gpu_matrix_jacobi(lina_gpu_matrix* m, int precision, double omega, int sweeps, const void* b_dev,
                           void* x_dev, void* tmp_dev);
int lina_gpu_matrix_rows(const lina_gpu_matrix* m);
/* stored entries including the SELL-32 slice padding */
long lina_gpu_matrix_padded_entries(const lina_gpu_matrix* m);
/* column-index width the matrix's FP32 passes read: 16 or 32 (SELL-32), 0 for the lane-group CSR
   layout */
int lina_gpu_matrix_index_bits(const lina_gpu_matrix* m);

/* ILU(0) preconditioner on the GPU: factors as incomplete_LU_factorization produces them
   (LinA/linear_algebra.c:1952: L lower with diagonal, U upper with unit diagonal), applied by
   forward and backward solves with one thread per row in level order, each row waiting only for
   the rows it needs. */
typedef struct lina_gpu_ilu lina_gpu_ilu;
int lina_gpu_ilu_create(int n, const int* Lptr, const int* Lcol, const double* Lval, const int* Uptr,
                        const int* Ucol, const double* Uval, lina_gpu_ilu** out);
/* ILU(0) of A (CSR, sorted distinct columns) factorised on the GPU, bit-identical to the reference's
   incomplete_LU_factorization (row recurrences run in level order, each row waiting only for the rows
   it needs); LINA_GPU_ESETUP on a zero pivot */
int lina_gpu_ilu_create_from_matrix(int n, const int* rowptr, const int* col, const double* val, lina_gpu_ilu** out);
/* the factors of a handle from lina_gpu_ilu_create_from_matrix on A's pattern (val[nnz]): L_ij where
   j <= i, U_ij where j > i (U's unit diagonal is not stored) */
int lina_gpu_ilu_factor_values(const lina_gpu_ilu* h, double* val);
/* new values of A on the pattern of a handle from lina_gpu_ilu_create_from_matrix (val[nnz]; host
   pointer, or device pointer with LINA_PCG_DEVICE_PTRS): the factors are recomputed on the device
   (bit-identical to a new handle), the level schedules and the pattern are kept;
   LINA_GPU_ESETUP on a zero pivot */
int lina_gpu_ilu_refactor(lina_gpu_ilu* h, const double* val, int flags);
int lina_gpu_ilu_destroy(lina_gpu_ilu* h);
/* The failure path of the bounded waits in the ILU kernels, made to happen: one thread waits for a
   device flag that nothing sets, up to limit_us microseconds (1 to 1,000,000).  Returns
   LINA_GPU_ECUDA with the error text a timed-out solve gives, and the time waited in *waited_us;
   the device stays usable.  For tests of the library's failure handling. */
int lina_gpu_wait_probe(int limit_us, double* waited_us);
int lina_gpu_ilu_levels(const lina_gpu_ilu* h, int* nlev_L, int* nlev_U);
/* z = U^-1 L^-1 r (device vectors, FP64); LINA_PREC_MIXED solves in FP32 */
int lina_gpu_ilu_apply(lina_gpu_ilu* h, int precision, const double* r_dev, double* z_dev);
/* device time of one application (forward and backward triangular solve, without the precision
   conversions of lina_gpu_ilu_apply): reps applications to a right-hand side of ones, timed with CUDA
   events on the handle's stream; *ms_per_apply = milliseconds per application */
int lina_gpu_ilu_time_apply(lina_gpu_ilu* h, int precision, int reps, double* ms_per_apply);

/* BiCGStab (BiCGStab_solve, LinA/BiCGStab.c:115-198) on device vectors with A a device matrix and
   the ILU(0) preconditioner (or none if ilu is NULL); stops when ||r|| / ||r0|| <= tol.
   flags: LINA_PCG_DEVICE_PTRS, LINA_PCG_USE_X0; ilu_precision selects the precision of the ILU solves. */
int lina_gpu_bicgstab(lina_gpu_matrix* A, lina_gpu_ilu* ilu, int ilu_precision, const double* b, double* x,
                      double tol, int max_iter, int flags, lina_gpu_solve_info* info);

/* Restarted GMRES (the gmres entry point, LinA/gmres.c:308) on A with a right preconditioner: the
   ILU(0) `ilu`, one V-cycle of `amg` from a zero guess, or none (both NULL); precon_precision
   selects the ILU solves' precision.  Solves A B_r y = b from the given y; y is the preconditioned
   iterate, unless flags hold LINA_GMRES_APPLY_PRECON, in which case y receives x = B_r y.
   Stops when ||b - A B_r y|| / ||b - A B_r y_0|| <= tol, tested at every step (check_each_iter)
   or at restarts every i_max steps; the step limit max_iter is tested at restarts.  info->iterations
   = Arnoldi steps, info->rel_residual = the last residual quotient.  Returns 0, LINA_GPU_ENOCONV
   (step limit) or LINA_GPU_EBREAKDOWN (singular Hessenberg system). */
#define LINA_GMRES_APPLY_PRECON 128
int lina_gpu_gmres(lina_gpu_matrix* A, lina_gpu_ilu* ilu, lina_gpu_amg* amg, int precon_precision, const double* b,
                   double* y, double tol, int i_max, int max_iter, int check_each_iter, int flags,
                   lina_gpu_solve_info* info);

/* C = A B (A: n rows, columns indexing the nb rows of B; CSR, FP64) on the GPU with the
   reference's sparse_product semantics (LinA/linear_algebra.c:186-222): row i starts as (i, 0.0),
   products of nonzero factors accumulate per column in A's and B's stored order, zeros are deleted
   (an emptied row keeps (i, 0.0)) -- bit-identical to the reference.  The AMG setup and recompute
   of device hierarchies form their Galerkin products R (A P) with it.  Host arrays; *nnz receives
   the entry count; with capacity 0 only *nnz is computed (C pointers may be NULL), otherwise
   capacity must hold nnz entries.  LINA_GPU_ECUDA also when a row has more than 512 distinct
   columns (the device table's bound). */
int lina_gpu_spgemm(int n, int ncols_b, const int* Ap, const int* Ac, const double* Av, int nb, const int* Bp,
                    const int* Bc, const double* Bv, long capacity, int* Cp, int* Cc, double* Cv, long* nnz);

/* reflective_newton (LinA/reflective_newton.c:660) on min x.A.x/2 + x.b, lower <= x <= upper, for a
   CSR Hessian and host arrays: the drop-in set-up done for the caller (the reference's default
   parameters, every unknown bounded, local solver `solver` -- RN_GPU_BICGSTAB_ILU keeps the Newton
   solves on the device -- with BiCGStab tolerance bi_eps).  x holds the start and receives the
   minimiser; returns the Newton steps or a negative LINA_GPU_E* code. */
int lina_gpu_reflective_newton_csr(int n, const int* ptr, const int* col, const double* val, const double* b,
                                   const double* lower, const double* upper, double* x, int solver, int max_iter,
                                   double eps, double bi_eps);

/* ---------------------------------------------------------------------------------------------
   Adjoint gradient of P1 plane-strain elasticity with a per-element Young's modulus (no reference
   counterpart; the reference's solvers applied to get_transpose(A), LinA/linear_algebra.c:1290,
   are its oracle).
   forward : A(E) = sum_e E_e Khat_e assembled on the GPU (Khat_e: the element stiffness with unit
             modulus), Dirichlet dofs eliminated symmetrically (identity rows, known values lifted
             into b), A u = b solved by AMG-PCG, L = 1/2 sum_s (u[sensor_dof_s] - target_s)^2.
   backward: A^T lambda = dL/du with the same hierarchy (A is symmetric by construction, so the
             transposed solve is the same operator), then dL/dE_e = -lambda_e^T Khat_e u_e per
             element (lambda_e: the element's six adjoint values, zero on Dirichlet dofs).
   Dof numbering: node k -> k (x), n_nodes + k (y), the reference's block ordering. */
/* P1 (linear triangle) assembly on the GPU, straight into CSR: the scalar Laplacian (one unknown
   per node; FEM2D's set_matrix_Aij_11_2D with insert_A_bbV_a, FEM2D/FEM2D.c:5949, :4728) or
   plane-strain elasticity (two per node, block ordering [x of all nodes, y of all nodes]), each
   element's matrix scaled by a per-element coefficient (conductivity, Young's modulus).  The
   pattern holds every pair of nodes sharing a triangle (both components for elasticity); Dirichlet
   dofs are eliminated symmetrically (identity rows, known values lifted into b).  Every stored
   entry sums its element contributions in element order with each product and sum rounded on its
   own, so the device values equal the host ones bit for bit.  No reference counterpart for the
   elimination: the reference resets rows only (Crack/crack.c:6445). */
#define LINA_P1_LAPLACE 1
#define LINA_P1_ELASTIC 2
typedef struct lina_gpu_p1 lina_gpu_p1;
typedef struct lina_gpu_p1_problem {
    int kind;                 /* LINA_P1_LAPLACE or LINA_P1_ELASTIC                     */
    int n_nodes, n_elems;
    const double* xy;         /* 2 per node                                              */
    const int* tri;           /* 3 node indices per element                              */
    double nu;                /* Poisson's ratio (LINA_P1_ELASTIC)                       */
    int n_fixed;
    const int* fixed_dof;     /* Dirichlet dofs: component * n_nodes + node              */
    const double* fixed_val;
} lina_gpu_p1_problem;
int lina_gpu_p1_create(const lina_gpu_p1_problem* p, lina_gpu_p1** out);
/* assemble with the per-element coefficients coef[n_elems] (host; device with LINA_PCG_DEVICE_PTRS):
   the matrix values and the right-hand side stay on the device */
int lina_gpu_p1_assemble(lina_gpu_p1* h, const double* coef, int flags);
int lina_gpu_p1_sizes(const lina_gpu_p1* h, int* n, long* nnz);
/* host copies of the pattern, the values and b of the last assembly (any pointer may be NULL) */
int lina_gpu_p1_download(lina_gpu_p1* h, int* rowptr, int* col, double* val, double* b);
/* the device arrays of the last assembly (owned by the handle): values on the pattern of rowptr/col,
   e.g. for lina_gpu_amg_update_values(..., LINA_PCG_DEVICE_PTRS) */
int lina_gpu_p1_device(lina_gpu_p1* h, const double** val_dev, const double** b_dev);
int lina_gpu_p1_destroy(lina_gpu_p1* h);
/* the same assembly on the host (rowptr[n+1], col[nnz], val[nnz], b[n]; *nnz alone when rowptr is
   NULL) */
int lina_gpu_p1_assemble_host(const lina_gpu_p1_problem* p, const double* coef, int* rowptr, int* col, double* val,
                              double* b, long* nnz);

typedef struct lina_gpu_elastic lina_gpu_elastic;
typedef struct lina_gpu_elastic_problem {
    int n_nodes;
    int n_elems;
    const double* xy;          /* [2*n_nodes] x0, y0, x1, y1, ...                         */
    const int* tri;            /* [3*n_elems] node indices of each triangle               */
    double nu;                 /* Poisson's ratio (plane strain)                          */
    int n_fixed;
    const int* fixed_dof;      /* [n_fixed] Dirichlet dofs, distinct                      */
    const double* fixed_val;   /* [n_fixed] their values                                  */
    int n_sensors;
    const int* sensor_dof;     /* [n_sensors] observed dofs, distinct, not Dirichlet      */
    const double* target;      /* [n_sensors] observed values                             */
} lina_gpu_elastic_problem;

#define LINA_ELASTIC_RECOMPUTE 64  /* forward: rebuild the coarse levels for the new matrix
                                      (AMG_recompute_coarse_matrices) instead of keeping them */

/* builds the pattern, the per-entry element contributions and the AMG hierarchy of A(young)
   (young: host array of n_elems moduli); opt as for lina_gpu_amg_create */
int lina_gpu_elastic_create(const lina_gpu_elastic_problem* p, const double* young,
                            const lina_gpu_amg_options* opt, lina_gpu_elastic** out);
/* forward pass for the moduli `young` (n_elems); u (2*n_nodes) and loss may be NULL.
   flags: LINA_PCG_DEVICE_PTRS (young and u on the device), LINA_PCG_USE_X0 (start from the
   previous forward solution), LINA_ELASTIC_RECOMPUTE.  Stops at ||b - A u|| / ||b|| <= tol. */
int lina_gpu_elastic_forward(lina_gpu_elastic* h, const double* young, double tol, int max_iter, int flags,
                             double* u, double* loss, lina_gpu_solve_info* info);
/* backward pass at the last forward solution: grad (n_elems) = dL/dE, lambda (2*n_nodes) may be
   NULL; flags: LINA_PCG_DEVICE_PTRS */
int lina_gpu_elastic_backward(lina_gpu_elastic* h, double tol, int max_iter, int flags, double* grad,
                              double* lambda, lina_gpu_solve_info* info);
/* sizes of the assembled system, and the current system copied to the host (NULL skips) */
int lina_gpu_elastic_sizes(const lina_gpu_elastic* h, int* n, long* nnz);
int lina_gpu_elastic_system(lina_gpu_elastic* h, int* rowptr, int* col, double* val, double* b);
lina_gpu_amg* lina_gpu_elastic_amg(lina_gpu_elastic* h);
int lina_gpu_elastic_destroy(lina_gpu_elastic* h);
/* the same assembly on the host with the same arithmetic (bit-identical values); *nnz receives
   the entry count; with rowptr == NULL only *nnz is computed */
int lina_gpu_elastic_assemble_host(const lina_gpu_elastic_problem* p, const double* young, int* rowptr,
                                   int* col, double* val, double* b, long* nnz);

/* CUDA-event timing on the hierarchy's stream: elapsed milliseconds between begin and end */
int lina_gpu_timer_begin(lina_gpu_amg* h);
int lina_gpu_timer_end(lina_gpu_amg* h, double* ms);
/* number of kernels this library has launched since it was loaded */
unsigned long long lina_gpu_launches(void);

/* hierarchy inspection (host copies of what the GPU holds) */
int lina_gpu_amg_depth(const lina_gpu_amg* h);
/* column-index width the FP32 passes over a level's A, P and R read: 16 or 32 (SELL-32), 0 (lane-
   group CSR layout, or no such matrix) */
int lina_gpu_level_index_bits(const lina_gpu_amg* h, int level, int* A_bits, int* P_bits, int* R_bits);
int lina_gpu_level_sizes(const lina_gpu_amg* h, int level, int* n, long* nnz_A, long* nnz_P, long* nnz_R,
                         int* n_colours);
int lina_gpu_level_export(const lina_gpu_amg* h, int level, int* labels, int* A_ptr, int* A_col, double* A_val,
                          int* P_ptr, int* P_col, double* P_val, int* R_ptr, int* R_col, double* R_val);
int lina_gpu_level_colours(const lina_gpu_amg* h, int level, int* colour);
int lina_gpu_coarse_block_size(const lina_gpu_amg* h);
/* bytes held on the device by the hierarchy */
long lina_gpu_amg_device_bytes(const lina_gpu_amg* h);

/* result = a . b for device vectors of n FP64 values: single-pass grid reduction (block partial
   sums in device scratch memory, the last block adds them in a fixed order) */
int lina_gpu_dot(const double* a_dev, const double* b_dev, long n, double* result);
/* The same product for callers that cannot allocate device memory at the point of the call: an
   application that reserves the GPU's memory for its own pool when it starts, or a job under a hard
   device-memory quota, where a cudaMalloc during the computation fails or is not allowed.  No
   counterpart in the reference.  Its scratch is a 128 KB array defined in device memory by the
   library and kept on every GPU that loads it; n is limited to 33,554,432 elements (larger n returns
   LINA_GPU_EINVAL).  The call is synchronous: it waits for the library's own stream, runs on the
   legacy default stream and returns the result on the host, so it cannot be captured into a CUDA
   graph nor called from a host function enqueued on a stream.  Inputs the caller wrote on its own
   non-blocking streams must be complete (those streams synchronized) before the call.  All calls
   share the scratch array: calls that overlap on the GPU race.  The first call on a device looks up
   the array's address and keeps it; make it before any stream capture, and do not use this entry
   point after a cudaDeviceReset. */
int lina_gpu_dot_noalloc(const double* a_dev, const double* b_dev, long n, double* result);

/* device memory helpers so that callers need no CUDA runtime of their own */
void* lina_gpu_malloc(size_t bytes);
int lina_gpu_free(void* p);
int lina_gpu_memcpy_h2d(void* dst, const void* src, size_t bytes);
int lina_gpu_memcpy_d2h(void* dst, const void* src, size_t bytes);
int lina_gpu_synchronize(void);
void* lina_gpu_malloc_host(size_t bytes);   /* pinned host memory */
int lina_gpu_free_host(void* p);
int lina_gpu_device_count(void);
int lina_gpu_set_device(int device);   /* select the GPU for hierarchies created afterwards */
/* storage layout of matrices uploaded afterwards: 0 automatic (SELL-32 thread-per-row for levels of
   100k rows or more, CSR with a lane group per row otherwise), 1 SELL-32 always, 2 CSR lane groups
   always (group size chosen from the mean row length), 3..6 CSR lane groups of 4, 8, 16 or 32 lanes */
int lina_gpu_set_layout(int layout);
/* interior levels of at most max_rows rows (default 24576; a block's copy of x allows up to 49152
   rows in FP32 and 24576 in FP64) run each multicolour-SOR V-cycle step
   (pre: x = 0, the sweeps, the residual and the restriction; post: the prolongation and the sweeps)
   as one launch of a thread-block cluster, with cluster barriers between the colours, instead of one
   launch per colour and step; the results are bit-identical.  0 turns this off.  Takes effect for
   solves issued afterwards (a hierarchy's captured solve graph keeps the choice it was captured with). */
int lina_gpu_set_fused_rows(int max_rows);
/* damped Jacobi: levels of at most max_entries stored entries (and the rows above) run each V-cycle step
   as one cluster launch, two copies of x in shared memory (default 0 = never: measured slower than the
   separate launches on GB300); the results are those of the separate launches, bit for bit */
int lina_gpu_set_fused_jacobi_entries(long max_entries);
/* segmented batches created afterwards: run the multicolour-SOR step of concatenated levels as one
   cluster per group of whole systems (at most the fused-rows limit each); default 0 = off (measured
   slower than one launch per colour on GB300).  The sweeps equal the colour launches'; residuals and
   transfers sum rows in lane-group order (separate FP32 launches on levels of 20,000 rows or more use the
   quad layout's stored order), so results agree to rounding. */
int lina_gpu_set_fused_groups(int on);
/* hierarchies created (or loaded) afterwards time every level below the finest (at least 2,000 rows,
   at most 50M stored entries) in
   each candidate layout at upload (one thread per row, or 4, 8 or 16 lanes per row), 5 smoother sweeps
   plus a residual in their precision, and keep the fastest (default 0 = the fixed layout rule; segmented
   batches always tune).  The choice depends on timings, so two hierarchies of one matrix may differ in
   layout and hence in rounding.  LINA_SETUP_TIMING prints the times. */
int lina_gpu_set_autotune(int on);
/* 16 (default): SELL-32 matrices with long rows (at least 24 stored entries per row on average)
   uploaded afterwards also get 16-bit column indices, a 15-bit offset from one of two bases per
   slice of 32 rows, where every slice's columns fit two such windows; FP32 passes read those (2
   bytes less per stored entry), FP64 passes the int columns.  32: int columns only.  The results
   are identical. */
int lina_gpu_set_sell_index_bits(int bits);
/* 1 (default): SELL-32 matrices in natural row order uploaded afterwards (with 16-bit indices enabled)
   also get the quad layout, in which every lane holds four consecutive entries of its row (one 16-byte
   value load and one 8-byte index load), and their FP32 passes read it; 0: FP32 passes read the
   one-entry SELL-32 layout.  The results are identical. */
int lina_gpu_set_sell_quads(int on);
/* 1 (default): the solve's kernels are launched with programmatic dependent launch (each kernel waits
   for the previous grid before touching memory, and its blocks are scheduled while that grid drains);
   0: ordinary stream order.  Takes effect for launches issued afterwards (a hierarchy's captured solve
   graph keeps the choice it was captured with).  The results are identical. */
int lina_gpu_set_pdl(int on);
/* Device bytes that one hierarchy or matrix handle may allocate (0, the default: no limit).  An allocation
   that would exceed it fails as a failed cudaMalloc does: the call returns LINA_GPU_ECUDA with the reason
   in lina_gpu_last_error(), frees what the handle holds, and the device stays usable.  For callers with a
   fixed memory budget, and for tests of the failure paths. */
int lina_gpu_set_device_memory_limit(long bytes);

/* Dense inverse of a row-major m x m matrix in device memory, in place, by blocked Gauss-Jordan
   elimination without pivoting (the elimination order of the reference's dense LU,
   LinA/linear_algebra.c:2909, so it exists exactly when that factorisation does).  method selects the
   arithmetic of the rank-32 updates, which carry 2 m^3 flops: LINA_DENSE_SIMT on the FP64 CUDA cores,
   LINA_DENSE_DMMA on the FP64 tensor cores (mma.sync m8n8k4).  *ms (may be NULL) receives the device
   time.  LINA_GPU_ESETUP on a zero pivot.  The coarsest AMG block is inverted this way at set-up and
   recompute when it has at least the rows set by lina_gpu_set_coarse_inverse (default 256, SIMT);
   smaller blocks are inverted on the host. */
#define LINA_DENSE_SIMT 0
#define LINA_DENSE_DMMA 1
int lina_gpu_dense_inverse(int m, double* a_dev, int method, double* ms);
/* coarsest blocks of min_rows rows or more are inverted on the GPU with method (0: always on the host);
   hierarchies created or recomputed afterwards */
int lina_gpu_set_coarse_inverse(int min_rows, int method);

const char* lina_gpu_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* LINA_GPU_H */
