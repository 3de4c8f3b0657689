/*
 * lina_port.c - CPU restatement of the reference LinA solve phase (ORACLE;
 * see lina_port.h for what it covers and where each piece comes from).
 *
 * Plain C over CSR arrays.  Row sums run in stored column order like the
 * reference's row loops; loops over rows are split across OpenMP threads
 * where the reference's result does not depend on the order (SpMV, Jacobi,
 * one colour of multicolour SOR); lexicographic SOR stays serial.
 */
#include "lina_port.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define MAXL 32
#define LBL_UNDECIDED 0
#define LBL_ISOLATED 3

typedef struct {
    int n, nc;
    int *ptr, *col;
    double* val;
} csr_t;

typedef struct {
    int n;
    csr_t A, P, R;
    int* labels;
    int ncol;
    int* cptr;
    int* crows;
    double *x, *t, *b, *r;
} level_t;

struct port_amg {
    int depth, smoother, nu, nu_finest;
    double omega;
    level_t lv[MAXL];
    /* coarsest: dense no-pivot LU of the rows with more than one nonzero */
    int m;
    int* brows;
    int* inblock;
    double* LU; /* m x m, unit lower L below the diagonal, U on and above */
    double* diag;
    double* work;
    double* isoinv; /* finest level: 1/(first nonzero) of isolated rows */
};

static void csr_copy(csr_t* d, int n, int nc, const int* ptr, const int* col, const double* val) {
    d->n = n;
    d->nc = nc;
    int nnz = ptr[n];
    d->ptr = (int*)malloc((n + 1) * sizeof(int));
    d->col = (int*)malloc((nnz > 0 ? nnz : 1) * sizeof(int));
    d->val = (double*)malloc((nnz > 0 ? nnz : 1) * sizeof(double));
    memcpy(d->ptr, ptr, (n + 1) * sizeof(int));
    memcpy(d->col, col, nnz * sizeof(int));
    memcpy(d->val, val, nnz * sizeof(double));
}

static void csr_free(csr_t* d) {
    free(d->ptr);
    free(d->col);
    free(d->val);
    memset(d, 0, sizeof *d);
}

port_amg* port_amg_new(int depth, int smoother, double omega, int nu, int nu_finest) {
    if (depth < 1 || depth > MAXL) return NULL;
    port_amg* h = (port_amg*)calloc(1, sizeof(port_amg));
    h->depth = depth;
    h->smoother = smoother;
    h->omega = omega;
    h->nu = nu;
    h->nu_finest = nu_finest;
    return h;
}

int port_amg_set_level(port_amg* h, int l, int n, const int* A_ptr, const int* A_col, const double* A_val,
                       const int* labels, const int* P_ptr, const int* P_col, const double* P_val,
                       const int* R_ptr, const int* R_col, const double* R_val, int nc) {
    if (!h || l < 0 || l >= h->depth) return -1;
    level_t* L = &h->lv[l];
    L->n = n;
    csr_copy(&L->A, n, n, A_ptr, A_col, A_val);
    if (l > 0) {
        L->labels = (int*)malloc(n * sizeof(int));
        memcpy(L->labels, labels, n * sizeof(int));
        csr_copy(&L->P, n, nc, P_ptr, P_col, P_val);
        csr_copy(&L->R, nc, n, R_ptr, R_col, R_val);
    }
    L->x = (double*)calloc(n, sizeof(double));
    L->t = (double*)calloc(n, sizeof(double));
    L->b = (double*)calloc(n, sizeof(double));
    L->r = (double*)calloc(n, sizeof(double));
    return 0;
}

/* greedy first-fit colouring of {(i,j): a_ij != 0 or a_ji != 0, i != j} */
static int colouring(const csr_t* A, int* colour) {
    int n = A->n;
    int* tptr = (int*)calloc(n + 1, sizeof(int));
    for (int i = 0; i < n; i++)
        for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
            int j = A->col[p];
            if (j != i && j < n && A->val[p] != 0.0) tptr[j + 1]++;
        }
    for (int i = 0; i < n; i++) tptr[i + 1] += tptr[i];
    int* tadj = (int*)malloc((tptr[n] + 1) * sizeof(int));
    int* fill = (int*)malloc((n + 1) * sizeof(int));
    memcpy(fill, tptr, n * sizeof(int));
    for (int i = 0; i < n; i++)
        for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
            int j = A->col[p];
            if (j != i && j < n && A->val[p] != 0.0) tadj[fill[j]++] = i;
        }
    int* mark = (int*)malloc((n + 2) * sizeof(int));
    for (int i = 0; i < n + 2; i++) mark[i] = -1;
    for (int i = 0; i < n; i++) colour[i] = -1;
    int ncol = 0;
    for (int i = 0; i < n; i++) {
        for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
            int j = A->col[p];
            if (j != i && j < n && A->val[p] != 0.0 && colour[j] >= 0) mark[colour[j]] = i;
        }
        for (int p = tptr[i]; p < tptr[i + 1]; p++)
            if (colour[tadj[p]] >= 0) mark[colour[tadj[p]]] = i;
        int c = 0;
        while (mark[c] == i) c++;
        colour[i] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    free(mark);
    free(fill);
    free(tadj);
    free(tptr);
    return ncol;
}

int port_amg_colouring(const port_amg* h, int l, int* colour) {
    if (!h || l < 0 || l >= h->depth) return -1;
    return colouring(&h->lv[l].A, colour);
}

static double csr_diag(const csr_t* A, int i) {
    for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++)
        if (A->col[p] == i) return A->val[p];
    return 0.0;
}

int port_amg_finalize(port_amg* h) {
    for (int l = 1; l < h->depth; l++) {
        level_t* L = &h->lv[l];
        int* colour = (int*)malloc((L->n > 0 ? L->n : 1) * sizeof(int));
        L->ncol = colouring(&L->A, colour);
        L->cptr = (int*)calloc(L->ncol + 1, sizeof(int));
        L->crows = (int*)malloc((L->n > 0 ? L->n : 1) * sizeof(int));
        for (int i = 0; i < L->n; i++) L->cptr[colour[i] + 1]++;
        for (int c = 0; c < L->ncol; c++) L->cptr[c + 1] += L->cptr[c];
        int* fill = (int*)malloc((L->ncol + 1) * sizeof(int));
        memcpy(fill, L->cptr, L->ncol * sizeof(int));
        for (int i = 0; i < L->n; i++) L->crows[fill[colour[i]]++] = i;
        free(fill);
        free(colour);
    }
    /* coarsest: sub_convert_sparse_to_array + LU_factorzation, no pivoting */
    level_t* C = &h->lv[0];
    int n = C->n;
    h->inblock = (int*)calloc(n, sizeof(int));
    h->brows = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
    h->diag = (double*)calloc(n, sizeof(double));
    int* map = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
    int m = 0;
    for (int i = 0; i < n; i++) {
        int cnt = 0;
        for (int p = C->A.ptr[i]; p < C->A.ptr[i + 1]; p++)
            if (C->A.val[p] != 0.0) cnt++;
        h->diag[i] = csr_diag(&C->A, i);
        if (cnt > 1) {
            map[i] = m;
            h->brows[m++] = i;
            h->inblock[i] = 1;
        } else {
            map[i] = -1;
        }
    }
    h->m = m;
    h->LU = (double*)calloc((size_t)m * m + 1, sizeof(double));
    h->work = (double*)calloc(m + 1, sizeof(double));
    double* M = h->LU;
    for (int I = 0; I < m; I++) {
        int i = h->brows[I];
        for (int p = C->A.ptr[i]; p < C->A.ptr[i + 1]; p++) {
            int J = map[C->A.col[p]];
            if (J >= 0) M[(size_t)I * m + J] = C->A.val[p];
        }
    }
    free(map);
    for (int k = 0; k < m; k++) {
        double piv = M[(size_t)k * m + k];
        if (piv == 0.0) return -2;
#pragma omp parallel for schedule(static)
        for (int i = k + 1; i < m; i++) {
            double f = M[(size_t)i * m + k] / piv;
            M[(size_t)i * m + k] = f;
            if (f != 0.0)
                for (int j = k + 1; j < m; j++) M[(size_t)i * m + j] -= f * M[(size_t)k * m + j];
        }
    }
    /* isolated rows of the finest level */
    if (h->depth > 1) {
        level_t* F = &h->lv[h->depth - 1];
        h->isoinv = (double*)calloc(F->n, sizeof(double));
        for (int i = 0; i < F->n; i++)
            if (F->labels[i] == LBL_ISOLATED)
                for (int p = F->A.ptr[i]; p < F->A.ptr[i + 1]; p++)
                    if (F->A.val[p] != 0.0) {
                        h->isoinv[i] = 1.0 / F->A.val[p];
                        break;
                    }
    }
    return 0;
}

int port_amg_level_info(const port_amg* h, int l, int* n, long* nnz_A, long* nnz_P, long* nnz_R) {
    if (!h || l < 0 || l >= h->depth) return -1;
    const level_t* L = &h->lv[l];
    *n = L->n;
    *nnz_A = L->A.ptr ? L->A.ptr[L->n] : 0;
    *nnz_P = (l > 0 && L->P.ptr) ? L->P.ptr[L->n] : 0;
    *nnz_R = (l > 0 && L->R.ptr) ? L->R.ptr[L->R.n] : 0;
    return 0;
}

static void csr_out(const csr_t* m, int* ptr, int* col, double* val) {
    if (!m->ptr) return;
    if (ptr) memcpy(ptr, m->ptr, (m->n + 1) * sizeof(int));
    if (col) memcpy(col, m->col, m->ptr[m->n] * sizeof(int));
    if (val) memcpy(val, m->val, m->ptr[m->n] * sizeof(double));
}

int port_amg_level_export(const port_amg* h, int l, int* labels, int* A_ptr, int* A_col, double* A_val,
                          int* P_ptr, int* P_col, double* P_val, int* R_ptr, int* R_col, double* R_val) {
    if (!h || l < 0 || l >= h->depth) return -1;
    const level_t* L = &h->lv[l];
    csr_out(&L->A, A_ptr, A_col, A_val);
    if (l > 0) {
        if (labels) memcpy(labels, L->labels, L->n * sizeof(int));
        csr_out(&L->P, P_ptr, P_col, P_val);
        csr_out(&L->R, R_ptr, R_col, R_val);
    }
    return 0;
}

void port_amg_free(port_amg* h) {
    if (!h) return;
    for (int l = 0; l < h->depth; l++) {
        level_t* L = &h->lv[l];
        csr_free(&L->A);
        csr_free(&L->P);
        csr_free(&L->R);
        free(L->labels);
        free(L->cptr);
        free(L->crows);
        free(L->x);
        free(L->t);
        free(L->b);
        free(L->r);
    }
    free(h->brows);
    free(h->inblock);
    free(h->LU);
    free(h->diag);
    free(h->work);
    free(h->isoinv);
    free(h);
}

/* ------------------------------------------------------------- kernels */
static void spmv(const csr_t* A, const double* x, double* y) { /* sparse_mult, linear_algebra.c:134 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < A->n; i++) {
        double s = 0.0;
        for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) s += A->val[p] * x[A->col[p]];
        y[i] = s;
    }
}

void port_spmv(const port_amg* h, int l, const double* x, double* y) { spmv(&h->lv[l].A, x, y); }

/* one row of AMG_SOR_smoother (Multigrid.c:1353-1362) reading x */
static inline double sor_row(const csr_t* A, int i, const double* F, const double* x, double w) {
    double sum = F[i];
    int diag = -1;
    for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
        int j = A->col[p];
        if (j != i)
            sum -= A->val[p] * x[j];
        else
            diag = p;
    }
    double a = (diag >= 0) ? A->val[diag] : 0.0;
    return (1. - w) * x[i] + w * sum / a;
}

static void smooth(port_amg* h, level_t* L, const double* F, double* x, int iter) {
    const csr_t* A = &L->A;
    const double w = h->omega;
    for (int k = 0; k < iter; k++) {
        if (h->smoother == PORT_SMOOTHER_JACOBI) {
            memcpy(L->t, x, L->n * sizeof(double));
#pragma omp parallel for schedule(static)
            for (int i = 0; i < L->n; i++) {
                if (L->labels && L->labels[i] == LBL_UNDECIDED) continue;
                x[i] = sor_row(A, i, F, L->t, w);
            }
        } else if (h->smoother == PORT_SMOOTHER_MC_SOR) {
            for (int c = 0; c < L->ncol; c++) {
#pragma omp parallel for schedule(static)
                for (int q = L->cptr[c]; q < L->cptr[c + 1]; q++) {
                    int i = L->crows[q];
                    if (L->labels && L->labels[i] == LBL_UNDECIDED) continue;
                    x[i] = sor_row(A, i, F, x, w);
                }
            }
        } else {
            for (int i = 0; i < L->n; i++) {
                if (L->labels && L->labels[i] == LBL_UNDECIDED) continue;
                x[i] = sor_row(A, i, F, x, w);
            }
        }
    }
}

/* AMG_Direct_solver with the LU factors (Multigrid.c:1450-1455) */
static void coarse_solve(port_amg* h, const double* F, double* X) {
    level_t* C = &h->lv[0];
    int m = h->m;
    double* y = h->work;
    for (int i = 0; i < C->n; i++)
        if (!h->inblock[i]) X[i] = F[i] / h->diag[i];
    for (int I = 0; I < m; I++) {
        double s = F[h->brows[I]];
        const double* row = h->LU + (size_t)I * m;
        for (int J = 0; J < I; J++) s -= row[J] * y[J];
        y[I] = s;
    }
    for (int I = m - 1; I >= 0; I--) {
        double s = y[I];
        const double* row = h->LU + (size_t)I * m;
        for (int J = I + 1; J < m; J++) s -= row[J] * y[J];
        y[I] = s / row[I];
    }
    for (int I = 0; I < m; I++) X[h->brows[I]] = y[I];
}

/* AMG_V_cycle (Multigrid.c:1536-1580); X holds the initial guess */
static void vcycle(port_amg* h, int l, const double* F, double* X) {
    if (l == 0) {
        coarse_solve(h, F, X);
        return;
    }
    level_t* L = &h->lv[l];
    level_t* C = &h->lv[l - 1];
    int nu = (l == h->depth - 1) ? h->nu_finest : h->nu;
    smooth(h, L, F, X, nu);
    spmv(&L->A, X, L->r); /* R = F - A X (linear_map with fac -1) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < L->n; i++) L->r[i] = F[i] - L->r[i];
    spmv(&L->R, L->r, C->b);
    memset(C->x, 0, C->n * sizeof(double));
    vcycle(h, l - 1, C->b, C->x);
    spmv(&L->P, C->x, L->t); /* X += P e (linear_map with fac 1) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < L->n; i++) X[i] += L->t[i];
    smooth(h, L, F, X, nu);
}

void port_vcycle(port_amg* h, const double* r, double* z) {
    int l = h->depth - 1;
    level_t* F = &h->lv[l];
    memset(z, 0, F->n * sizeof(double));
    if (h->isoinv)
        for (int i = 0; i < F->n; i++)
            if (h->isoinv[i] != 0.0) z[i] = r[i] * h->isoinv[i];
    vcycle(h, l, r, z);
}

static double dot(const double* a, const double* b, int n) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

int port_pcg(port_amg* h, const double* B, double* X, double tol, int max_iter, int stop_rule, double max_seconds,
             double* pcg_res) {
    level_t* F = &h->lv[h->depth - 1];
    const csr_t* A = &F->A;
    int n = F->n;
    double t0 = omp_get_wtime();
    double hn = sqrt(dot(B, B, n));
    if (hn == 0) hn = 1;
    double* b = (double*)malloc(n * sizeof(double));
    double* R = (double*)malloc(n * sizeof(double));
    double* Z = (double*)malloc(n * sizeof(double));
    double* P = (double*)malloc(n * sizeof(double));
    double* Q = (double*)malloc(n * sizeof(double));
    for (int i = 0; i < n; i++) {
        b[i] = B[i] * (1.0 / hn);
        X[i] *= 1.0 / hn;
    }
    spmv(A, X, Q);
    for (int i = 0; i < n; i++) R[i] = b[i] - Q[i];
    port_vcycle(h, R, Z);
    double r0 = (stop_rule == 0) ? sqrt(dot(Z, Z, n)) : sqrt(dot(b, b, n));
    int it = 0;
    double s = 0, s_old = 0, r = r0;
    if (r0 != 0) {
        int have_z = 1;
        do {
            if (!have_z) port_vcycle(h, R, Z);
            have_z = 0;
            s_old = s;
            s = dot(R, Z, n);
            if (it > 0) {
                double beta = s / s_old;
                for (int i = 0; i < n; i++) P[i] = beta * P[i] + Z[i];
            } else {
                memcpy(P, Z, n * sizeof(double));
            }
            spmv(A, P, Q);
            double a = s / dot(P, Q, n);
            for (int i = 0; i < n; i++) {
                X[i] += a * P[i];
                R[i] -= a * Q[i];
            }
            r = sqrt(dot(R, R, n));
            it++;
            if (max_seconds > 0 && omp_get_wtime() - t0 > max_seconds) break;
        } while (r / r0 > tol && it < max_iter);
        if (pcg_res) {
            port_vcycle(h, R, Z);
            *pcg_res = sqrt(dot(Z, Z, n)) / r0;
        }
    }
    for (int i = 0; i < n; i++) X[i] *= hn;
    free(b);
    free(R);
    free(Z);
    free(P);
    free(Q);
    return it;
}

/* ILU(0) of A (CSR, sorted distinct columns) on A's pattern: incomplete_LU_factorization
   (LinA/linear_algebra.c:1952-1982) with row_times_row (:1795-1818).  f_p = L_ij for j <= i,
   U_ij for j > i; the sums run over ascending k where (i, k) and (k, j) are in the pattern and
   start at 0.  Returns 1, or 0 on a zero (or absent) pivot L_ii of a row with entries right of
   the diagonal, as the reference does. */
static int find_col(const int* col, int lo, int hi, int j) {
    hi--;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (col[mid] == j) return mid;
        if (col[mid] < j)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return -1;
}

int port_ilu0(int n, const int* ptr, const int* col, const double* a, double* f) {
    int* ustart = (int*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    if (!ustart) return -1;
    int ok = 1;
    for (int i = 0; i < n && ok; i++) {
        int r0 = ptr[i], r1 = ptr[i + 1];
        int split = r1;
        for (int p = r0; p < r1; p++)
            if (col[p] > i) {
                split = p;
                break;
            }
        ustart[i] = split;
        double d = 0.0;
        for (int p = r0; p < r1; p++) {
            int j = col[p];
            int jmax = j <= i ? j - 1 : i - 1;
            double s = 0.0;
            for (int q = r0; q < r1 && col[q] <= jmax; q++) {
                int k = col[q];
                int pos = find_col(col, ustart[k], ptr[k + 1], j);
                if (pos >= 0) s += f[q] * f[pos];
            }
            double v = a[p] - s;
            if (j <= i) {
                f[p] = v;
                if (j == i) d = v;
            } else {
                if (d == 0.0) {
                    ok = 0;
                    break;
                }
                f[p] = v / d;
            }
        }
    }
    free(ustart);
    return ok;
}

/* ------------------------------------------------------------------ BiCGStab with ILU(0)
   The reference's BiCGStab_solve (BiCGStab.c:115-198) with the product sparse_mult (linear_algebra.c:134:
   each row's products summed in stored order) and the preconditioner of its ILU test drivers: x = y, then
   L_triang_invert and U_triang_invert (linear_algebra.c:2008-2043) with the factors of
   incomplete_LU_factorization (:1952).  The reference's L row holds the columns j <= i in ascending order
   with the diagonal last, its U row (built transposed, then transposed back) the unit diagonal first and
   the columns j > i ascending; the solves subtract in that order, so on CSR rows with ascending columns
   the sums here are the reference's.  Vector operations are the reference's serial loops (scalar,
   vector_add, scalar_mult, euklid_norm: linear_algebra.c:256-316). */
static void bi_mult(int n, const int* ptr, const int* col, const double* a, const double* y, double* x) {
    for (int i = 0; i < n; i++) {
        double sum = 0;
        for (int p = ptr[i]; p < ptr[i + 1]; p++) sum += a[p] * y[col[p]];
        x[i] = sum;
    }
}

static double bi_scalar(const double* x, const double* y, int n) {
    double r = 0;
    for (int i = 0; i < n; i++) r = r + x[i] * y[i];
    return r;
}

static void bi_add(double* x, const double* y, double factor, int n) {
    for (int i = 0; i < n; i++) x[i] += factor * y[i];
}

static void bi_ilu_apply(int n, const int* ptr, const int* col, const double* f, const double* y, double* x,
                         double* tmp) {
    /* L_triang_invert: x_i = (y_i - sum_{j<i} L_ij x_j) / L_ii */
    for (int i = 0; i < n; i++) tmp[i] = y[i];
    for (int i = 0; i < n; i++) {
        double sum = tmp[i], diag = 0;
        for (int p = ptr[i]; p < ptr[i + 1] && col[p] <= i; p++) {
            if (col[p] != i)
                sum -= f[p] * x[col[p]];
            else
                diag = f[p];
        }
        x[i] = sum / diag;
    }
    /* U_triang_invert: unit diagonal first, then the columns j > i */
    for (int i = 0; i < n; i++) tmp[i] = x[i];
    for (int i = n - 1; i >= 0; i--) {
        double sum = tmp[i];
        for (int p = ptr[i]; p < ptr[i + 1]; p++)
            if (col[p] > i) sum -= f[p] * x[col[p]];
        x[i] = sum / 1.0;
    }
}

int port_bicgstab_ilu(int n, const int* ptr, const int* col, const double* a, const double* f, const double* b,
                      double* x, double eps, int max_iter, int use_ilu, double* rel_out) {
    const double default_eps = 1e-10;
    double* w = (double*)calloc((size_t)(n > 0 ? n : 1) * 10, sizeof(double));
    if (!w) return -1;
    double *S = w, *PS = w + n, *PP = w + 2 * (size_t)n, *APP = w + 3 * (size_t)n, *APS = w + 4 * (size_t)n;
    double *R = w + 5 * (size_t)n, *R0 = w + 6 * (size_t)n, *P = w + 7 * (size_t)n, *T = w + 8 * (size_t)n;
    bi_mult(n, ptr, col, a, x, R);
    bi_add(R, b, -1., n);
    for (int i = 0; i < n; i++) R[i] *= -1;
    memcpy(R0, R, (size_t)n * sizeof(double));
    memcpy(P, R, (size_t)n * sizeof(double));
    int iter = 0;
    const double r0 = sqrt(bi_scalar(R, R, n));
    double r = r0;
    if (r0 != 0) {
        do {
            if (use_ilu)
                bi_ilu_apply(n, ptr, col, f, P, PP, T);
            else
                memcpy(PP, P, (size_t)n * sizeof(double));
            bi_mult(n, ptr, col, a, PP, APP);
            const double h = bi_scalar(R, R0, n);
            const double t = bi_scalar(APP, R0, n);
            if (t == 0) {
                (void)default_eps;
                break;
            }
            const double alpha = h / t;
            memcpy(S, R, (size_t)n * sizeof(double));
            bi_add(S, APP, -alpha, n);
            if (use_ilu)
                bi_ilu_apply(n, ptr, col, f, S, PS, T);
            else
                memcpy(PS, S, (size_t)n * sizeof(double));
            bi_mult(n, ptr, col, a, PS, APS);
            const double s = bi_scalar(APS, APS, n);
            if (s == 0) break;
            const double omega = bi_scalar(APS, S, n) / s;
            bi_add(x, PP, alpha, n);
            bi_add(x, PS, omega, n);
            memcpy(R, S, (size_t)n * sizeof(double));
            bi_add(R, APS, -omega, n);
            const double beta = bi_scalar(R, R0, n) * alpha / (h * omega);
            bi_add(P, APP, -omega, n);
            for (int i = 0; i < n; i++) P[i] *= beta;
            bi_add(P, R, 1., n);
            r = sqrt(bi_scalar(R, R, n));
            iter++;
        } while (r / r0 > eps && iter <= max_iter);
    }
    if (rel_out) *rel_out = r0 != 0 ? r / r0 : 0.0;
    free(w);
    return iter;
}
