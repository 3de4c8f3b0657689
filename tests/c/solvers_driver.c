/*
 * solvers_driver.c - a caller of LinA's gmres, Newton_solver and active_set_solver, written the
 * way FEM2D/FEM.c and Crack/crack.c call the reference library, compiled against the headers in
 * include/ and linked with the GB300 library.  Used by tests/test_gmres_newton.py.
 *
 * usage: solvers_driver <mode> <in.bin> <out.bin>
 *   in.bin : int32 n, int32 nnz, int32 p0, int32 p1, int32 p2, float64 q0, float64 q1,
 *            int32 indptr[n+1], int32 indices[nnz], float64 data[nnz], float64 b[n],
 *            float64 x0[n], float64 lower[n], float64 upper[n]
 *   modes  : "gmres"       gmres with PCG_mult and PCG_preconlr after PCG_default(A, L, U) (the
 *                          library's own product and ILU(0)); p0 = i_max, p1 = maxiter,
 *                          p2 = check each step, q0 = tol
 *            "gmres-host"  the same with the caller's own host product and ILU callbacks
 *            "newton"      Newton_solver for A x + q1 x^3 = b from x0; p0 = mode (LARGE_SYSTEM /
 *                          SMALL_SYSTEM), p1 = GMRES i_max, p2 = Newton steps, q0 = eps
 *            "active"      active_set_solver with identity constraints lower <= x <= upper and
 *                          a dense-LU KKT solver; p0 = max_iter
 *            "active-gpu"  the same with the library's GMRES + ILU(0) KKT solver on the device
 *   out.bin: int32 r0, int32 r1, int32 r2, float64 d0, float64 x[n]
 *            gmres: iterations, rcode, nomatvec, precision;  newton: steps;
 *            active: iterations, final active count
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "GMRES_Newton.h"
#include "PCGS.h"
#include "itlin.h"
#include "linear_algebra.h"

static sparse_matrix *A = NULL, *L = NULL, *U = NULL;
static double cubic = 0.0;

static void host_matvec(int n, double* y, double* z) {
    double* r = sparse_mult(A, y);
    memcpy(z, r, n * sizeof(double));
    free(r);
}

static void host_ilu(int n, double* z, double* w) {
    memcpy(w, z, n * sizeof(double));
    L_triang_invert(L, w);
    U_triang_invert(U, w);
}

static double reaction(double* X, int i, int size) {
    (void)size;
    double s = 0;
    for (int j = 0; j < A->Len[i]; j++) s += A->Values[i][j] * X[A->Indices[i][j]];
    return s + cubic * X[i] * X[i] * X[i];
}

static int dense_lu(sparse_matrix* M, double* X, double* b) {
    sparse_matrix* l = sparse_zero(M->size);
    sparse_matrix* u = sparse_zero(M->size);
    complete_LU_factorization(M, l, u);
    memcpy(X, b, M->size * sizeof(double));
    L_triang_invert(l, X);
    U_triang_invert(u, X);
    free_sparse(l);
    free_sparse(u);
    return 1;
}

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    FILE* f = fopen(argv[2], "rb");
    if (!f) return 2;
    int hdr[5];
    double q[2];
    if (fread(hdr, sizeof(int), 5, f) != 5 || fread(q, sizeof(double), 2, f) != 2) return 2;
    int n = hdr[0], nnz = hdr[1];
    int* ptr = malloc((n + 1) * sizeof(int));
    int* col = malloc(nnz * sizeof(int));
    double* val = malloc(nnz * sizeof(double));
    double* b = malloc(n * sizeof(double));
    double* x = malloc(n * sizeof(double));
    double* lo = malloc(n * sizeof(double));
    double* up = malloc(n * sizeof(double));
    if (fread(ptr, sizeof(int), n + 1, f) != (size_t)(n + 1) || fread(col, sizeof(int), nnz, f) != (size_t)nnz ||
        fread(val, sizeof(double), nnz, f) != (size_t)nnz || fread(b, sizeof(double), n, f) != (size_t)n ||
        fread(x, sizeof(double), n, f) != (size_t)n || fread(lo, sizeof(double), n, f) != (size_t)n ||
        fread(up, sizeof(double), n, f) != (size_t)n)
        return 2;
    fclose(f);
    A = sparse_zero(n);
    for (int i = 0; i < n; i++)
        for (int p = ptr[i]; p < ptr[i + 1]; p++) {
            if (col[p] == i)
                set_sparse(A, val[p], i, i);
            else
                insert_sparse(A, val[p], i, col[p]);
        }

    int out_i[3] = {0, 0, 0};
    double out_d = 0.0;
    if (!strcmp(argv[1], "gmres") || !strcmp(argv[1], "gmres-host")) {
        L = sparse_zero(n);
        U = sparse_zero(n);
        incomplete_LU_factorization(A, L, U);
        struct ITLIN_OPT opt;
        struct ITLIN_INFO info;
        memset(&opt, 0, sizeof opt);
        memset(&info, 0, sizeof info);
        opt.tol = q[0];
        opt.i_max = hdr[2];
        opt.maxiter = hdr[3];
        opt.termcheck = hdr[4] ? CheckEachIter : CheckOnRestart;
        opt.errorlevel = None;
        if (!strcmp(argv[1], "gmres")) {
            PCG_default(A, L, U);
            gmres(n, x, PCG_mult, (PRECON*)PCG_preconlr, NULL, b, &opt, &info);
        } else {
            gmres(n, x, host_matvec, host_ilu, NULL, b, &opt, &info);
        }
        out_i[0] = info.iter;
        out_i[1] = info.rcode;
        out_i[2] = info.nomatvec;
        out_d = info.precision;
    } else if (!strcmp(argv[1], "newton")) {
        cubic = q[1];
        Newton_set_function(reaction);
        Newton_set_inhomo(b, n);
        Newton_GMRES_options(hdr[3], 1000, 1e-10);
        Newton_set_range(n, lo, up);
        out_i[0] = Newton_solver(A, x, hdr[4], q[0], hdr[2], -1.0);
    } else if (!strcmp(argv[1], "active") || !strcmp(argv[1], "active-gpu")) {
        sparse_matrix* B = sparse_identity(n);
        ass_info* info = NULL;
        out_i[0] = active_set_solver(A, x, b, B, lo, up, !strcmp(argv[1], "active") ? dense_lu : LinA_gpu_general_solver,
                                     hdr[2], POS_DEFINITE, ASS_DEFAULT, &info);
        out_i[1] = info->active_size;
        free_ass_info(&info);
        free_sparse(B);
    } else {
        return 2;
    }
    FILE* o = fopen(argv[3], "wb");
    if (!o) return 2;
    fwrite(out_i, sizeof(int), 3, o);
    fwrite(&out_d, sizeof(double), 1, o);
    fwrite(x, sizeof(double), n, o);
    fclose(o);
    return 0;
}
