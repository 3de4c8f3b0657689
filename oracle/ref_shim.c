/*
 * ref_shim.c - test-infrastructure driver around the reference LinA library.
 *
 * This file is ORACLE code: it is compiled together with the reference's own
 * LinA sources (LinA/*.c, built unmodified from where they lie) into
 * oracle/_ref/libLinA_ref.so by oracle/Makefile.  Only tests and the CPU
 * baseline leg of bench.py load it, and only to produce the values the GPU
 * library is checked against.  It calls the reference exclusively through its
 * public API (linear_algebra.h, Multigrid.h, PCGS.h, BiCGStab.h).
 *
 * What it adds:
 *  - CSR <-> row-list conversion (the reference's matrix type is
 *    LinA/linear_algebra.h:29-34);
 *  - accessors for the AMG hierarchy (LinA/Multigrid.h:45-70);
 *  - a PCG driver whose preconditioner is exactly one V-cycle from a zero
 *    guess (AMG_solve with max_iter 1, LinA/Multigrid.c:1863-1931);
 *  - two smoothers installed through the reference's own plug-in
 *    AMG_set_smoother (LinA/Multigrid.c:1967): damped Jacobi and multicolour
 *    SOR (greedy first-fit colouring of the symmetric nonzero graph), which
 *    are the GPU smoothers' algorithms;
 *  - a switch that makes malloc return zero-filled memory (glibc M_PERTURB),
 *    so that the reference's read of an uninitialised array
 *    (Importance_2nd, LinA/Multigrid.c:566) is deterministic.
 */
#include <fcntl.h>
#include <malloc.h>
#include <string.h>
#include <unistd.h>

#include "BiCGStab.h"
#include "Multigrid.h"
#include "PCGS.h"
#include "linear_algebra.h"

/* ---------------------------------------------------------------- stdout */
static int saved_stdout = -1;

void rs_silence(int on) {
    fflush(stdout);
    if (on && saved_stdout < 0) {
        saved_stdout = dup(1);
        int fd = open("/dev/null", O_WRONLY);
        dup2(fd, 1);
        close(fd);
    } else if (!on && saved_stdout >= 0) {
        dup2(saved_stdout, 1);
        close(saved_stdout);
        saved_stdout = -1;
    }
}

void rs_malloc_zero(void) { mallopt(M_PERTURB, 255); }

/* ------------------------------------------------------------ conversions */
sparse_matrix* rs_from_csr(int n, const int* indptr, const int* indices, const double* data) {
    sparse_matrix* A = (sparse_matrix*)malloc(sizeof(sparse_matrix));
    A->size = n;
    A->Len = (int*)malloc(n * sizeof(int));
    A->Values = (double**)malloc(n * sizeof(double*));
    A->Indices = (int**)malloc(n * sizeof(int*));
    for (int i = 0; i < n; i++) {
        int len = indptr[i + 1] - indptr[i];
        if (len == 0) { /* the reference's empty row holds one explicit (i, 0.0) */
            A->Len[i] = 1;
            A->Values[i] = (double*)malloc(sizeof(double));
            A->Indices[i] = (int*)malloc(sizeof(int));
            A->Values[i][0] = 0.0;
            A->Indices[i][0] = i;
            continue;
        }
        A->Len[i] = len;
        A->Values[i] = (double*)malloc(len * sizeof(double));
        A->Indices[i] = (int*)malloc(len * sizeof(int));
        memcpy(A->Values[i], data + indptr[i], len * sizeof(double));
        memcpy(A->Indices[i], indices + indptr[i], len * sizeof(int));
    }
    return A;
}

void rs_free(sparse_matrix* A) {
    if (A) { free_sparse(A); }
}

int rs_size(const sparse_matrix* A) { return A ? A->size : 0; }

long rs_nnz(const sparse_matrix* A) {
    long s = 0;
    if (!A) return 0;
    for (int i = 0; i < A->size; i++) s += A->Len[i];
    return s;
}

void rs_to_csr(const sparse_matrix* A, int* indptr, int* indices, double* data) {
    long p = 0;
    indptr[0] = 0;
    for (int i = 0; i < A->size; i++) {
        memcpy(indices + p, A->Indices[i], A->Len[i] * sizeof(int));
        memcpy(data + p, A->Values[i], A->Len[i] * sizeof(double));
        p += A->Len[i];
        indptr[i + 1] = (int)p;
    }
}

/* ---------------------------------------------------------------- AMG */
amg_system_info* rs_amg_setup(sparse_matrix* A, int dof, int depth, int sm, int aggr_sm, int coarsening) {
    AMG_print_info(NO);
    return AMG_setup(A, dof, depth, sm, aggr_sm, coarsening, STAND_ALONE, DIRECT, NULL, NULL);
}

int rs_amg_depth(const amg_system_info* I) { return I->depth; }
int rs_amg_fine_size(const amg_system_info* I, int level) { return I->Fine_sizes[level]; }
int rs_amg_coarse_size(const amg_system_info* I, int level) { return I->Coarse_sizes[level]; }
sparse_matrix* rs_amg_A(amg_system_info* I, int level) { return I->Coarse_A[level]; }
sparse_matrix* rs_amg_P(amg_system_info* I, int level) { return I->Prolongation[level]; }
sparse_matrix* rs_amg_R(amg_system_info* I, int level) { return I->Restriction[level]; }
sparse_matrix* rs_amg_L(amg_system_info* I, int level) { return I->L[level]; }
sparse_matrix* rs_amg_U(amg_system_info* I, int level) { return I->U[level]; }
sparse_matrix* rs_amg_signs(amg_system_info* I) { return I->Signs; }
const int* rs_amg_labels(const amg_system_info* I, int level) { return I->Coarsening[level]; }

void rs_amg_free(amg_system_info* I) {
    if (I) {
        AMG_free_data(I);
        free(I);
    }
}

void rs_amg_recompute(amg_system_info* I, sparse_matrix* A) { AMG_recompute_coarse_matrices(I, A); }

/* --------------------------------------------------------- smoothers (oracle) */
/* greedy first-fit colouring of the symmetric graph {(i,j): a_ij != 0 or a_ji != 0, i != j} */
static const sparse_matrix* col_key = NULL;
static int col_n = 0;
static int* col_of = NULL;
static int col_count = 0;
static int* col_rows = NULL;   /* rows grouped by colour, increasing row index inside a colour */
static int* col_ptr = NULL;

int rs_greedy_colouring(const sparse_matrix* A, int* colour) {
    int n = A->size;
    /* transpose adjacency (nonzero off-diagonal entries) */
    int* tcount = (int*)calloc(n + 1, sizeof(int));
    for (int i = 0; i < n; i++)
        for (int k = 0; k < A->Len[i]; k++) {
            int j = A->Indices[i][k];
            if (j != i && j < n && A->Values[i][k] != 0.0) tcount[j + 1]++;
        }
    for (int i = 0; i < n; i++) tcount[i + 1] += tcount[i];
    int* tadj = (int*)malloc((tcount[n] + 1) * sizeof(int));
    int* fill = (int*)calloc(n, sizeof(int));
    for (int i = 0; i < n; i++)
        for (int k = 0; k < A->Len[i]; k++) {
            int j = A->Indices[i][k];
            if (j != i && j < n && A->Values[i][k] != 0.0) tadj[tcount[j] + fill[j]++] = i;
        }
    int ncol = 0;
    int* mark = (int*)malloc((n + 2) * sizeof(int));
    for (int i = 0; i < n + 2; i++) mark[i] = -1;
    for (int i = 0; i < n; i++) colour[i] = -1;
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < A->Len[i]; k++) {
            int j = A->Indices[i][k];
            if (j != i && j < n && A->Values[i][k] != 0.0 && colour[j] >= 0) mark[colour[j]] = i;
        }
        for (int k = tcount[i]; k < tcount[i + 1]; k++) {
            int j = tadj[k];
            if (colour[j] >= 0) mark[colour[j]] = i;
        }
        int c = 0;
        while (mark[c] == i) c++;
        colour[i] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    free(mark);
    free(fill);
    free(tadj);
    free(tcount);
    return ncol;
}

static void ensure_colouring(const sparse_matrix* A) {
    if (col_key == A && col_n == A->size) return;
    free(col_of);
    free(col_rows);
    free(col_ptr);
    col_n = A->size;
    col_key = A;
    col_of = (int*)malloc(col_n * sizeof(int));
    col_count = rs_greedy_colouring(A, col_of);
    col_ptr = (int*)calloc(col_count + 1, sizeof(int));
    col_rows = (int*)malloc(col_n * sizeof(int));
    for (int i = 0; i < col_n; i++) col_ptr[col_of[i] + 1]++;
    for (int c = 0; c < col_count; c++) col_ptr[c + 1] += col_ptr[c];
    int* fill = (int*)calloc(col_count, sizeof(int));
    for (int i = 0; i < col_n; i++) col_rows[col_ptr[col_of[i]] + fill[col_of[i]]++] = i;
    free(fill);
}

void rs_forget_colouring(void) { col_key = NULL; }

static double smoother_omega = 1.0;

/* multicolour SOR: colours in increasing order, SOR update of Multigrid.c:1345-1364 per row */
static void rs_multicolour_sor(sparse_matrix* A, double* F, double* Sol, int* Label, double alpha, int fix,
                               int iter, int deg_freedom) {
    (void)alpha;
    (void)deg_freedom;
    ensure_colouring(A);
    double w = smoother_omega;
    for (int k = 0; k < iter; k++)
        for (int c = 0; c < col_count; c++)
            for (int p = col_ptr[c]; p < col_ptr[c + 1]; p++) {
                int i = col_rows[p];
                if (Label[i] == fix) continue;
                double sum = F[i], diag = 0.0;
                for (int j = 0; j < A->Len[i]; j++) {
                    int ind = A->Indices[i][j];
                    if (ind != i) sum -= A->Values[i][j] * Sol[ind];
                    else diag = A->Values[i][j];
                }
                Sol[i] = (1.0 - w) * Sol[i] + w * sum / diag;
            }
}

/* damped Jacobi with the same per-row update */
static void rs_damped_jacobi(sparse_matrix* A, double* F, double* Sol, int* Label, double alpha, int fix, int iter,
                             int deg_freedom) {
    (void)alpha;
    (void)deg_freedom;
    int n = A->size;
    double w = smoother_omega;
    double* Old = (double*)malloc(n * sizeof(double));
    for (int k = 0; k < iter; k++) {
        memcpy(Old, Sol, n * sizeof(double));
        for (int i = 0; i < n; i++) {
            if (Label[i] == fix) continue;
            double sum = F[i], diag = 0.0;
            for (int j = 0; j < A->Len[i]; j++) {
                int ind = A->Indices[i][j];
                if (ind != i) sum -= A->Values[i][j] * Old[ind];
                else diag = A->Values[i][j];
            }
            Sol[i] = (1.0 - w) * Old[i] + w * sum / diag;
        }
    }
    free(Old);
}

/* kind: 0 reference lexicographic SOR, 1 reference parallel Jacobi, 2 damped Jacobi, 3 multicolour SOR */
void rs_set_smoother(int kind, double omega) {
    smoother_omega = omega;
    AMG_set_SOR_relaxation_coeff(omega);
    switch (kind) {
        case 1: AMG_set_smoother(AMG_parallel_Jacobi_smoother); break;
        case 2: AMG_set_smoother(rs_damped_jacobi); break;
        case 3: AMG_set_smoother(rs_multicolour_sor); break;
        default: AMG_set_smoother(AMG_SOR_smoother);
    }
}

/* ------------------------------------------------------------------ PCG */
static amg_system_info* pcg_amg = NULL;

static int rs_precon_one_vcycle(int n, double* R, double* Z) {
    memset(Z, 0, n * sizeof(double));
    AMG_solve(pcg_amg, R, Z, NULL);
    return 1;
}

/* pcg (LinA/PCGS.c:163-233) on A with a one-V-cycle zero-guess AMG preconditioner */
int rs_pcg_amg(amg_system_info* I, sparse_matrix* A, double* x, double* b, double tol, int max_iter, double* pcg_res) {
    pcg_amg = I;
    AMG_print_info(NO);
    AMG_set_max_iter(1);
    AMG_set_eps(0.0);
    PCG_default(A, NULL, NULL);
    PCG_set_precon(rs_precon_one_vcycle);
    int it = pcg(x, b, A->size, tol, max_iter);
    if (pcg_res) *pcg_res = get_pcg_residuum();
    return it;
}

/* AMG_solve as the reference runs it (V-cycles until eps or max_iter) */
int rs_amg_solve(amg_system_info* I, double* F, double* X, double eps, int max_iter) {
    AMG_print_info(NO);
    AMG_set_eps(eps);
    AMG_set_max_iter(max_iter);
    return AMG_solve(I, F, X, NULL);
}

/* one V-cycle from a zero guess (the preconditioner application) */
void rs_vcycle_zero(amg_system_info* I, double* R, double* Z) {
    pcg_amg = I;
    AMG_print_info(NO);
    AMG_set_max_iter(1);
    AMG_set_eps(0.0);
    rs_precon_one_vcycle(I->Fine_sizes[I->depth - 1], R, Z);
}

/* ------------------------------------------------------------ elementary */
void rs_spmv(sparse_matrix* A, const double* x, double* y) {
    double* r = sparse_mult(A, (double*)x);
    memcpy(y, r, A->size * sizeof(double));
    free(r);
}

sparse_matrix* rs_product(sparse_matrix* A, sparse_matrix* B) { return sparse_product(A, B); }
sparse_matrix* rs_transpose(sparse_matrix* A, int new_size) { return get_transpose(A, new_size); }

int rs_ilu(sparse_matrix* A, sparse_matrix** L, sparse_matrix** U) {
    *L = sparse_zero(A->size);
    *U = sparse_zero(A->size);
    return incomplete_LU_factorization(A, *L, *U);
}

void rs_ilu_apply(sparse_matrix* L, sparse_matrix* U, double* x) {
    L_triang_invert(L, x);
    U_triang_invert(U, x);
}

/* the reference's own AMG preconditioner path: PCG_default + PCG_set_AMG_preconditioner
   (LinA/PCGS.c:29, :118-129) + pcg; the smoother installed by rs_set_smoother stays in place */
int rs_pcg_stock_amg(sparse_matrix* A, int dof, int depth, double omega, double* x, double* b, double tol,
                     int max_iter, double* pcg_res) {
    PCG_default(A, NULL, NULL);
    PCG_set_AMG_preconditioner(A, dof, depth);
    AMG_set_SOR_relaxation_coeff(omega);
    smoother_omega = omega;
    int it = pcg(x, b, A->size, tol, max_iter);
    if (pcg_res) *pcg_res = get_pcg_residuum();
    return it;
}

/* AMG_solve from a zero guess to eps with at most max_iter V-cycles */
int rs_amg_solve_fresh(amg_system_info* I, double* F, double* X, double eps, int max_iter) {
    AMG_print_info(NO);
    AMG_set_eps(eps);
    AMG_set_max_iter(max_iter);
    return AMG_solve(I, F, X, NULL);
}

/* BiCGStab_solve (LinA/BiCGStab.c:115) with A as the product and ILU(0) of A as the preconditioner */
static sparse_matrix *bi_A = NULL, *bi_L = NULL, *bi_U = NULL;
static void bi_matvec(int n, double* y, double* x) {
    double* r = sparse_mult(bi_A, y);
    memcpy(x, r, n * sizeof(double));
    free(r);
}
static int bi_ilu(int n, double* y, double* x) {
    memcpy(x, y, n * sizeof(double));
    L_triang_invert(bi_L, x);
    U_triang_invert(bi_U, x);
    return 1;
}
int rs_bicgstab_ilu(sparse_matrix* A, double* x, double* b, double eps, int max_iter, int use_ilu) {
    bi_A = A;
    bi_L = sparse_zero(A->size);
    bi_U = sparse_zero(A->size);
    if (!incomplete_LU_factorization(A, bi_L, bi_U)) return -1;
    BI_set_mat_mult(bi_matvec);
    BI_set_precon(use_ilu ? bi_ilu : NULL);
    BI_set_eps(eps);
    BI_set_max_iter(max_iter);
    BI_print_info(NO);
    BI_set_stat("", "");
    int it = BiCGStab_solve(x, b, A->size);
    free_sparse(bi_L);
    free_sparse(bi_U);
    return it;
}

/* ---------------------------------------------------------- reflective Newton (reference) */
#include "reflective_newton.h"

static int rs_rn_local_bicgstab_ilu(sparse_matrix* M, double* X, double* b) {
    /* BiCGStab_solve with the ILU(0) of M (BI_eps, BI_max_iter as set by the caller) */
    bi_A = M;
    bi_L = sparse_zero(M->size);
    bi_U = sparse_zero(M->size);
    if (!incomplete_LU_factorization(M, bi_L, bi_U)) {
        free_sparse(bi_L);
        free_sparse(bi_U);
        return INDEFINITE;
    }
    BI_set_mat_mult(bi_matvec);
    BI_set_precon(bi_ilu);
    BI_print_info(NO);
    int it = BiCGStab_solve(X, b, M->size);
    free_sparse(bi_L);
    free_sparse(bi_U);
    return it < BI_get_max_iter() ? POSITIVE_DEFINITE : INDEFINITE;
}

/* minimise x.H.x/2 + x.b subject to lower <= x <= upper with reflective_newton
   (LinA/reflective_newton.c:660); solver 3 = RN_PCG (ILU-PCG), 5 = BiCGStab+ILU(0) through the
   local-solver slot.  Returns the Newton iterations; x holds the start on entry. */
/* The reference seeds its negative-curvature search with srand(time(NULL))
   (set_random_normal_vector, LinA/linear_algebra.c:4823-4828), its only use of time(): inside this
   library time() returns 1, so a run repeats and draws the start vector the GPU library draws. */
time_t time(time_t* t) {
    if (t) *t = 1;
    return 1;
}

/* the count of negative-curvature events of the last reflective_newton run (print_RN_statistics) */
int rs_rn_neg_curv(void) {
    char buf[4096];
    FILE* f = fmemopen(buf, sizeof buf, "w");
    if (!f) return -1;
    print_RN_statistics(f);
    fclose(f);
    buf[sizeof buf - 1] = 0;
    const char* key = "number of neg. curvature events: ";
    const char* p = strstr(buf, key);
    return p ? atoi(p + strlen(key)) : -1;
}

int rs_reflective_newton_qp(sparse_matrix* H, double* b, double* lower, double* upper, double* x, int solver,
                            int max_iter, double eps, double bi_eps) {
    int n = H->size;
    int* idx = get_all_indices(n);
    RN_print_info(RN_NO);
    RN_init_statistics();
    RN_set_params(max_iter, eps, 0.1, 0.9, 0.1, 250., 1., 0.6, 1.1, 1e-3, 1000.);
    set_RN_Hesse(H);
    set_RN_linear(b);
    set_RN_functional(NULL);
    RN_set_gradient(NULL);
    set_RN_constraints(idx, lower, upper, n);
    BI_set_eps(bi_eps);
    BI_set_max_iter(1000);
    BI_set_stat("", "");
    if (solver == RN_UMF)
        RN_set_local_solver(rs_rn_local_bicgstab_ilu);
    else {
        RN_set_local_solver(NULL);
        RN_set_solver(solver);
    }
    int it = reflective_newton(x);
    free(idx);
    return it;
}

/* ---------------------------------------------------------- gmres, Newton, active set (reference) */
#include "GMRES_Newton.h"
#include "itlin.h"
extern void gmres(int n, double* y, MATVEC* matvec, PRECON* preconr, PRECON* preconl, double* b,
                  struct ITLIN_OPT* opt, struct ITLIN_INFO* info);

static sparse_matrix *gm_A = NULL, *gm_L = NULL, *gm_U = NULL;
static void gm_matvec(int n, double* y, double* z) {
    double* r = sparse_mult(gm_A, y);
    memcpy(z, r, n * sizeof(double));
    free(r);
}
static void gm_ilu(int n, double* z, double* w) {
    memcpy(w, z, n * sizeof(double));
    L_triang_invert(gm_L, w);
    U_triang_invert(gm_U, w);
}

/* the reference gmres (LinA/gmres.c:308) on A y = b with the ILU(0) of A as right preconditioner
   (or none); y holds the start on entry and the preconditioned iterate on exit.
   out: iterations, rcode, nomatvec; precision */
int rs_gmres(sparse_matrix* A, double* y, double* b, double tol, int i_max, int maxiter, int check_each,
             int use_ilu, int* out, double* precision) {
    gm_A = A;
    gm_L = sparse_zero(A->size);
    gm_U = sparse_zero(A->size);
    if (use_ilu) incomplete_LU_factorization(A, gm_L, gm_U);
    struct ITLIN_OPT opt;
    struct ITLIN_INFO info;
    memset(&opt, 0, sizeof opt);
    memset(&info, 0, sizeof info);
    opt.tol = tol;
    opt.i_max = i_max;
    opt.maxiter = maxiter;
    opt.termcheck = check_each ? CheckEachIter : CheckOnRestart;
    opt.errorlevel = None;
    opt.monitorlevel = None;
    opt.datalevel = None;
    gmres(A->size, y, gm_matvec, use_ilu ? gm_ilu : NULL, NULL, b, &opt, &info);
    free_sparse(gm_L);
    free_sparse(gm_U);
    out[0] = info.iter;
    out[1] = info.rcode;
    out[2] = info.nomatvec;
    *precision = info.precision;
    return info.iter;
}

/* F_i(X) = (A X)_i + c X_i^3 on the pattern of A: a discretised nonlinear reaction-diffusion
   operator for the Newton solver tests */
static sparse_matrix* nw_A = NULL;
static double nw_c = 0.0;
static double nw_F(double* X, int i, int size) {
    double s = 0;
    for (int j = 0; j < nw_A->Len[i]; j++) s += nw_A->Values[i][j] * X[nw_A->Indices[i][j]];
    return s + nw_c * X[i] * X[i] * X[i];
}

/* Newton_solver (LinA/GMRES_Newton.c:212) for F(X) = B from X; mode LARGE_SYSTEM (ILU-GMRES with
   i_max, gmres_maxiter, gmres_tol) or SMALL_SYSTEM (sparse LU); returns the Newton steps */
int rs_newton(sparse_matrix* A, double c, double* B, double* X, int maxiter, double eps, int mode, int i_max,
              int gmres_maxiter, double gmres_tol) {
    nw_A = A;
    nw_c = c;
    Newton_set_function(nw_F);
    Newton_set_inhomo(B, A->size);
    Newton_GMRES_options(i_max, gmres_maxiter, gmres_tol);
    double* lo = malloc(A->size * sizeof(double));
    double* hi = malloc(A->size * sizeof(double));
    for (int i = 0; i < A->size; i++) lo[i] = -1e300, hi[i] = 1e300;
    Newton_set_range(A->size, lo, hi);
    free(lo);
    free(hi);
    return Newton_solver(A, X, maxiter, eps, mode, -1.0);
}

/* the dense-LU solver callback of the active-set tests */
static int as_dense_lu(sparse_matrix* M, double* X, double* b) {
    sparse_matrix* L = sparse_zero(M->size);
    sparse_matrix* U = sparse_zero(M->size);
    complete_LU_factorization(M, L, U);
    memcpy(X, b, M->size * sizeof(double));
    L_triang_invert(L, X);
    U_triang_invert(U, X);
    free_sparse(L);
    free_sparse(U);
    return 1;
}

/* active_set_solver (LinA/linear_algebra.c:4933) with B = identity: lower <= x <= upper, KKT
   systems solved by a dense LU; returns the active-set iterations, *active_size the final count */
int rs_active_set(sparse_matrix* A, double* x, double* b, double* lower, double* upper, int max_iter,
                  int* active_size) {
    sparse_matrix* B = sparse_identity(A->size);
    ass_info* info = NULL;
    int it = active_set_solver(A, x, b, B, lower, upper, as_dense_lu, max_iter, POS_DEFINITE, ASS_DEFAULT, &info);
    *active_size = info->active_size;
    free_ass_info(&info);
    free_sparse(B);
    return it;
}

/* ---------------------------------------------------------- full multigrid (reference) */
/* AMG_solve with the full-multigrid cycle structure (LinA/Multigrid.c:1582-1611, :1908) from X */
int rs_amg_fmg(amg_system_info* I, double* F, double* X) {
    AMG_print_info(NO);
    int old = I->AMG_cycle_structure;
    I->AMG_cycle_structure = FULL_AMG;
    int it = AMG_solve(I, F, X, NULL);
    I->AMG_cycle_structure = old;
    return it;
}
