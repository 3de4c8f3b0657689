/*
 * dropin_driver.c - a caller of the LinA API, written the way Crack/crack.c
 * and FEM2D call the reference library, compiled against the headers in include/ and
 * linked with the GB300 library.  Used by tests/test_dropin.py.
 *
 * usage: dropin_driver <mode> <in.bin> <out.bin>
 *   in.bin : int32 n, int32 nnz, int32 dof, int32 depth, int32 coarsening,
 *            int32 smoother (0 SOR, 1 parallel Jacobi, 2 damped Jacobi), float64 omega,
 *            int32 indptr[n+1], int32 indices[nnz], float64 data[nnz], float64 b[n]
 *   modes  : "vcycle-pcg"  pcg with a caller-defined preconditioner running one
 *                          V-cycle from a zero guess through AMG_solve
 *            "device-pcg"  PCG_default + PCG_set_AMG_data + PCG_AMG_vcycle_precon: the same
 *                          preconditioner as the library's, pcg on the device
 *            "device-pcg-clone"  the same with a copy of A as operator (host-driven loop)
 *            "stock"       PCG_default + PCG_set_AMG_preconditioner + pcg
 *            "amgsolve"    AMG_solve alone to 1e-8 (at most 200 V-cycles)
 *   out.bin: int32 iterations, float64 residuum, float64 x[n]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "BiCGStab.h"
#include "Multigrid.h"
#include "PCGS.h"
#include "linear_algebra.h"

static amg_system_info* amg = NULL;

static int vcycle_precon(int n, double* R, double* Z) {
    memset(Z, 0, n * sizeof(double));
    return AMG_solve(amg, R, Z, NULL);
}

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    FILE* f = fopen(argv[2], "rb");
    if (!f) return 2;
    int hdr[6];
    double omega;
    if (fread(hdr, sizeof(int), 6, f) != 6 || fread(&omega, sizeof(double), 1, f) != 1) return 2;
    int n = hdr[0], nnz = hdr[1], dof = hdr[2], depth = hdr[3], coarsening = hdr[4], smoother = hdr[5];
    int* ptr = malloc((n + 1) * sizeof(int));
    int* col = malloc(nnz * sizeof(int));
    double* val = malloc(nnz * sizeof(double));
    double* b = malloc(n * sizeof(double));
    if (fread(ptr, sizeof(int), n + 1, f) != (size_t)(n + 1) || fread(col, sizeof(int), nnz, f) != (size_t)nnz ||
        fread(val, sizeof(double), nnz, f) != (size_t)nnz || fread(b, sizeof(double), n, f) != (size_t)n)
        return 2;
    fclose(f);

    /* assemble the row-list matrix through the API, as FEM2D does */
    sparse_matrix* A = sparse_zero(n);
    for (int i = 0; i < n; i++)
        for (int p = ptr[i]; p < ptr[i + 1]; p++) {
            if (col[p] == i)
                set_sparse(A, val[p], i, i); /* the (i, 0.0) placeholder becomes the diagonal */
            else
                insert_sparse(A, val[p], i, col[p]);
        }

    AMG_print_info(NO);
    if (smoother == 1)
        AMG_set_smoother(AMG_parallel_Jacobi_smoother);
    else if (smoother == 2)
        AMG_set_smoother(AMG_damped_Jacobi_smoother);
    else
        AMG_set_smoother(AMG_SOR_smoother);

    double* x = zero_vector(n);
    int it = -1;
    double res = 0;
    if (!strcmp(argv[1], "vcycle-pcg")) {
        AMG_set_SOR_relaxation_coeff(omega);
        amg = AMG_setup(A, dof, depth, 2, 2, coarsening, STAND_ALONE, DIRECT, NULL, NULL);
        AMG_set_max_iter(1);
        AMG_set_eps(0.0);
        PCG_default(A, NULL, NULL);
        PCG_set_precon(vcycle_precon);
        it = pcg(x, b, n, 1e-8, 500);
        res = get_pcg_residuum();
        AMG_free_data(amg);
        free(amg);
    } else if (!strcmp(argv[1], "device-pcg") || !strcmp(argv[1], "device-pcg-clone")) {
        /* the library's zero-guess V-cycle preconditioner: the whole pcg loop runs on the device; with
           a copy of A as the operator the same preconditioner runs inside the host-driven loop */
        AMG_set_SOR_relaxation_coeff(omega);
        amg = AMG_setup(A, dof, depth, 2, 2, coarsening, STAND_ALONE, DIRECT, NULL, NULL);
        sparse_matrix* op = !strcmp(argv[1], "device-pcg") ? A : clone(A);
        PCG_default(op, NULL, NULL);
        PCG_set_AMG_data(amg);
        PCG_set_precon(PCG_AMG_vcycle_precon);
        it = pcg(x, b, n, 1e-8, 500);
        res = get_pcg_residuum();
        if (op != A) {
            free_sparse(op);
        }
        AMG_free_data(amg);
        free(amg);
    } else if (!strcmp(argv[1], "stock")) {
        PCG_default(A, NULL, NULL);
        PCG_set_AMG_preconditioner(A, dof, depth);
        AMG_set_SOR_relaxation_coeff(omega);
        it = pcg(x, b, n, 1e-8, 500);
        res = get_pcg_residuum();
    } else if (!strcmp(argv[1], "amgsolve")) {
        AMG_set_SOR_relaxation_coeff(omega);
        amg = AMG_setup(A, dof, depth, 2, 2, coarsening, STAND_ALONE, DIRECT, NULL, NULL);
        AMG_set_max_iter(200);
        AMG_set_eps(1e-8);
        it = AMG_solve(amg, b, x, NULL);
        res = matrix_residuum(A, x, b);
    } else {
        return 2;
    }
    FILE* o = fopen(argv[3], "wb");
    fwrite(&it, sizeof(int), 1, o);
    fwrite(&res, sizeof(double), 1, o);
    fwrite(x, sizeof(double), n, o);
    fclose(o);
    free_sparse(A);
    free(x);
    free(ptr);
    free(col);
    free(val);
    free(b);
    return it < 0 ? 1 : 0;
}
