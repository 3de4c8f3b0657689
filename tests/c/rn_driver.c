/*
 * rn_driver.c - a caller of LinA's reflective Newton minimiser, written the way
 * Crack/crack.c calls the reference library (set_RN_Hesse / set_RN_linear /
 * set_RN_constraints / RN_set_local_solver / reflective_newton), compiled
 * against the headers in include/ and linked with the GB300 library.  Used by
 * tests/test_reflective_newton.py.
 *
 * usage: rn_driver <mode> <in.bin> <out.bin>
 *   in.bin : int32 n, int32 nnz, int32 max_iter, float64 eps, float64 bi_eps,
 *            int32 indptr[n+1], int32 indices[nnz], float64 data[nnz],
 *            float64 b[n], float64 lower[n], float64 upper[n], float64 x0[n]
 *   modes  : "gpu"   RN_set_solver(RN_GPU_BICGSTAB_ILU): BiCGStab + ILU(0) on the device
 *            "umf"   RN_set_local_solver with a caller solver running BiCGStab_solve
 *            "spd"   RN_set_local_solver(LinA_gpu_spd_solver): AMG-PCG on the device
 *                    preconditioned by the ILU(0) of the local matrix (host triangular solves)
 *            "pcg"   RN_set_solver(RN_PCG): ILU-preconditioned pcg
 *   out.bin: int32 iterations, float64 x[n]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "BiCGStab.h"
#include "PCGS.h"
#include "linear_algebra.h"
#include "reflective_newton.h"

static sparse_matrix *loc_L = NULL, *loc_U = NULL;

static int ilu_precon(int n, double* Y, double* X) {
    memcpy(X, Y, n * sizeof(double));
    L_triang_invert(loc_L, X);
    U_triang_invert(loc_U, X);
    return 1;
}

/* the local solver of a caller: ILU(0) + BiCGStab on the scaled Newton matrix */
static int local_bicgstab_ilu(sparse_matrix* M, double* X, double* b) {
    loc_L = sparse_zero(M->size);
    loc_U = sparse_zero(M->size);
    int ok = incomplete_LU_factorization(M, loc_L, loc_U);
    int status = INDEFINITE;
    if (ok) {
        BI_set_mat_mult(RN_default_mat_mult);
        BI_set_precon(ilu_precon);
        int it = BiCGStab_solve(X, b, M->size);
        status = (it >= 0 && it < BI_get_max_iter()) ? POSITIVE_DEFINITE : INDEFINITE;
    }
    free_sparse(loc_L);
    free_sparse(loc_U);
    return status;
}

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    FILE* f = fopen(argv[2], "rb");
    if (!f) return 2;
    int hdr[3];
    double eps, bi_eps;
    if (fread(hdr, sizeof(int), 3, f) != 3 || fread(&eps, sizeof(double), 1, f) != 1 ||
        fread(&bi_eps, sizeof(double), 1, f) != 1)
        return 2;
    int n = hdr[0], nnz = hdr[1], max_iter = hdr[2];
    int* ptr = malloc((n + 1) * sizeof(int));
    int* col = malloc(nnz * sizeof(int));
    double* val = malloc(nnz * sizeof(double));
    double* b = malloc(n * sizeof(double));
    double* lo = malloc(n * sizeof(double));
    double* up = malloc(n * sizeof(double));
    double* x = malloc(n * sizeof(double));
    if (fread(ptr, sizeof(int), n + 1, f) != (size_t)(n + 1) || fread(col, sizeof(int), nnz, f) != (size_t)nnz ||
        fread(val, sizeof(double), nnz, f) != (size_t)nnz || fread(b, sizeof(double), n, f) != (size_t)n ||
        fread(lo, sizeof(double), n, f) != (size_t)n || fread(up, sizeof(double), n, f) != (size_t)n ||
        fread(x, sizeof(double), n, f) != (size_t)n)
        return 2;
    fclose(f);

    sparse_matrix* H = sparse_zero(n);
    for (int i = 0; i < n; i++)
        for (int p = ptr[i]; p < ptr[i + 1]; p++) {
            if (col[p] == i)
                set_sparse(H, val[p], i, i);
            else
                insert_sparse(H, val[p], i, col[p]);
        }
    int* idx = get_all_indices(n);

    RN_print_info(RN_NO);
    RN_init_statistics();
    RN_set_params(max_iter, eps, 0.1, 0.9, 0.1, 250., 1., 0.6, 1.1, 1e-3, 1000.);
    set_RN_Hesse(H);
    set_RN_linear(b);
    set_RN_functional(NULL);
    RN_set_gradient(NULL);
    set_RN_constraints(idx, lo, up, n);
    BI_set_eps(bi_eps);
    BI_set_max_iter(1000);
    BI_print_info(NO);
    if (!strcmp(argv[1], "gpu")) {
        RN_set_local_solver(NULL);
        RN_set_solver(RN_GPU_BICGSTAB_ILU);
    } else if (!strcmp(argv[1], "umf")) {
        RN_set_local_solver(local_bicgstab_ilu);
    } else if (!strcmp(argv[1], "spd")) {
        /* the library's AMG-PCG local solver in the slot crack.c fills with its UMFPACK wrapper */
        RN_set_local_solver(LinA_gpu_spd_solver);
    } else if (!strcmp(argv[1], "pcg")) {
        RN_set_local_solver(NULL);
        RN_set_solver(RN_PCG);
    } else {
        return 2;
    }
    int it = reflective_newton(x);

    FILE* o = fopen(argv[3], "wb");
    if (!o) return 2;
    fwrite(&it, sizeof(int), 1, o);
    fwrite(x, sizeof(double), n, o);
    fclose(o);
    free_sparse(H);
    free(idx);
    free(ptr);
    free(col);
    free(val);
    free(b);
    free(lo);
    free(up);
    free(x);
    return 0;
}
