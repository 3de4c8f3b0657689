// lina_api.cpp - the reference LinA C API (linear_algebra.h, Multigrid.h,
// PCGS.h, BiCGStab.h) implemented on top of the GB300 kernels.
//
// Callers keep their calls: matrices stay the reference's row-list
// sparse_matrix, solver settings stay file-scope state set through the same
// setter functions, and return values keep their meaning (iteration counts).
// What moves to the GPU:
//  - AMG_setup builds the hierarchy with the host setup that reproduces the
//    reference's (amg_host.cpp) and uploads it; AMG_solve runs its V-cycles on
//    the GPU (lina_gpu_amg_solve);
//  - pcg and BiCGStab_solve keep their vectors on the GPU; the library's own
//    operators (PCG_mult, PCG_AMG_precon, BI_AMG_precon) run there, and a
//    caller's own callbacks are called on host copies of the vectors.
// Matrix helpers (insertion, products on row lists) are host functions over
// the caller's data, exactly like the reference's.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "BiCGStab.h"
#include "amg_host.h"
#include "Multigrid.h"
#include "PCGS.h"
#include "reflective_newton.h"
#include <cuda_runtime.h>

#include "gpu_ops.h"
#include "lina_gpu.h"
#include "lina_internal.h"
#include "linear_algebra.h"

// ============================================================ row-list helpers
extern "C" {

int min(int a, int b) { return a < b ? a : b; }
int max(int a, int b) { return a > b ? a : b; }

double* zero_vector(int n) { return (double*)calloc(n > 0 ? n : 1, sizeof(double)); }

double* clone_vector(double* x, int n) {
    double* y = (double*)malloc((n > 0 ? n : 1) * sizeof(double));
    memcpy(y, x, n * sizeof(double));
    return y;
}

void copy_vector_to(double* x, double* y, int n) { memcpy(y, x, n * sizeof(double)); }

double scalar(double* x1, double* x2, int n) {
    double r = 0;
    for (int i = 0; i < n; i++) r = r + x1[i] * x2[i];
    return r;
}

double euklid_norm(double* x1, int n) { return sqrt(scalar(x1, x1, n)); }

void scalar_mult(double a, double* x, int n) {
    for (int i = 0; i < n; i++) x[i] *= a;
}

void vector_add(double* x, double* y, double factor, int n) {
    for (int i = 0; i < n; i++) x[i] += factor * y[i];
}

// insertion position in a sorted index list; *Flag = 1 if val is present (linear_algebra.c:1515)
int get_position(int* list, int size, int val, int* Flag) {
    *Flag = -1;
    if (size <= 0) return -1;
    int lo = 0, hi = size;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (list[mid] < val)
            lo = mid + 1;
        else
            hi = mid;
    }
    if (lo < size && list[lo] == val) *Flag = 1;
    return lo;
}

sparse_matrix* sparse_diagonal(double* d, int n) {
    sparse_matrix* r = (sparse_matrix*)malloc(sizeof(sparse_matrix));
    r->Values = (double**)malloc(n * sizeof(double*));
    r->Indices = (int**)malloc(n * sizeof(int*));
    r->Len = (int*)malloc(n * sizeof(int));
    for (int i = 0; i < n; i++) {
        r->Values[i] = (double*)malloc(sizeof(double));
        r->Indices[i] = (int*)malloc(sizeof(int));
        r->Values[i][0] = d[i];
        r->Indices[i][0] = i;
        r->Len[i] = 1;
    }
    r->size = n;
    return r;
}

sparse_matrix* sparse_zero(int length) {
    std::vector<double> z(length > 0 ? length : 1, 0.0);
    return sparse_diagonal(z.data(), length);
}

sparse_matrix* sparse_identity(int length) {
    std::vector<double> z(length > 0 ? length : 1, 1.0);
    return sparse_diagonal(z.data(), length);
}

sparse_matrix* clone(sparse_matrix* A) {
    int n = A->size;
    sparse_matrix* r = (sparse_matrix*)malloc(sizeof(sparse_matrix));
    r->size = n;
    r->Len = (int*)malloc(n * sizeof(int));
    r->Values = (double**)malloc(n * sizeof(double*));
    r->Indices = (int**)malloc(n * sizeof(int*));
    for (int i = 0; i < n; i++) {
        int len = A->Len[i];
        r->Len[i] = len;
        r->Values[i] = (double*)malloc((len > 0 ? len : 1) * sizeof(double));
        r->Indices[i] = (int*)malloc((len > 0 ? len : 1) * sizeof(int));
        memcpy(r->Values[i], A->Values[i], len * sizeof(double));
        memcpy(r->Indices[i], A->Indices[i], len * sizeof(int));
    }
    return r;
}

void Free_sparse(sparse_matrix* A) {
    lina::api::forget_device_matrix(A);  // a device copy cached for this matrix goes with it
    for (int i = 0; i < A->size; i++) {
        free(A->Values[i]);
        free(A->Indices[i]);
    }
    free(A->Len);
    free(A->Values);
    free(A->Indices);
}

void insert_element_at(sparse_matrix* A, double a, int i, int j, int pos) {
    int len = A->Len[i];
    A->Values[i] = (double*)realloc(A->Values[i], (len + 1) * sizeof(double));
    A->Indices[i] = (int*)realloc(A->Indices[i], (len + 1) * sizeof(int));
    memmove(A->Values[i] + pos + 1, A->Values[i] + pos, (len - pos) * sizeof(double));
    memmove(A->Indices[i] + pos + 1, A->Indices[i] + pos, (len - pos) * sizeof(int));
    A->Values[i][pos] = a;
    A->Indices[i][pos] = j;
    A->Len[i]++;
}

// removing the last entry of a row leaves (i, 0.0), as the reference does (linear_algebra.c:1161-1178)
void remove_element_at(sparse_matrix* A, int i, int pos) {
    int len = A->Len[i];
    if (len > 1) {
        memmove(A->Values[i] + pos, A->Values[i] + pos + 1, (len - pos - 1) * sizeof(double));
        memmove(A->Indices[i] + pos, A->Indices[i] + pos + 1, (len - pos - 1) * sizeof(int));
        A->Len[i]--;
    } else {
        A->Values[i][0] = 0.0;
        A->Indices[i][0] = i;
    }
}

int insert_sparse(sparse_matrix* A, double a, int i, int j) {
    int flag;
    int pos = get_position(A->Indices[i], A->Len[i], j, &flag);
    if (pos < 0) pos = 0;
    if (flag < 0)
        insert_element_at(A, a, i, j, pos);
    else
        A->Values[i][pos] += a;
    return pos;
}

void set_sparse(sparse_matrix* A, double a, int i, int j) {
    int flag;
    int pos = get_position(A->Indices[i], A->Len[i], j, &flag);
    if (pos < 0) pos = 0;
    if (flag < 0)
        insert_element_at(A, a, i, j, pos);
    else
        A->Values[i][pos] = a;
}

void remove_element(sparse_matrix* A, int i, int j) {
    int flag;
    int pos = get_position(A->Indices[i], A->Len[i], j, &flag);
    if (flag > 0) remove_element_at(A, i, pos);
}

void reset_row(sparse_matrix* A, int i) {
    free(A->Values[i]);
    free(A->Indices[i]);
    A->Values[i] = (double*)malloc(sizeof(double));
    A->Indices[i] = (int*)malloc(sizeof(int));
    A->Values[i][0] = 0.0;
    A->Indices[i][0] = i;
    A->Len[i] = 1;
}

void delete_zeros(sparse_matrix* A) {
    for (int i = 0; i < A->size; i++) {
        if (A->Len[i] <= 1) continue;
        int w = 0;
        for (int k = 0; k < A->Len[i]; k++)
            if (A->Values[i][k] != 0.0) {
                A->Values[i][w] = A->Values[i][k];
                A->Indices[i][w] = A->Indices[i][k];
                w++;
            }
        if (w == 0) {
            A->Values[i][0] = 0.0;
            A->Indices[i][0] = i;
            w = 1;
        }
        A->Len[i] = w;
    }
}

// removes the last zero entry of row i (linear_algebra.c:1905)
void remove_zero(sparse_matrix* A, int i) {
    int k = -1;
    for (int j = 0; j < A->Len[i]; j++)
        if (A->Values[i][j] == 0) k = j;
    if (k >= 0) remove_element_at(A, i, k);
}

void remove_zeros(sparse_matrix* A) {
    for (int i = 0; i < A->size; i++) remove_zero(A, i);
}

double get_matrix_element(sparse_matrix* A, int i, int j) {
    int flag;
    int pos = get_position(A->Indices[i], A->Len[i], j, &flag);
    return flag == 1 ? A->Values[i][pos] : 0.0;
}

double get_diag(sparse_matrix* A, int i) { return get_matrix_element(A, i, i); }

int write_sparse(sparse_matrix* A, char* path, char* name) {
    if (!A || !path || !name) return 0;
    std::string file = std::string(path) + "/" + name;
    FILE* f = fopen(file.c_str(), "wb");
    if (!f) return 0;
    const int n = A->size;
    bool ok = fwrite(&n, sizeof(int), 1, f) == 1 && (n == 0 || fwrite(A->Len, sizeof(int), n, f) == (size_t)n);
    for (int i = 0; ok && i < n; i++)
        ok = A->Len[i] == 0 || fwrite(A->Indices[i], sizeof(int), A->Len[i], f) == (size_t)A->Len[i];
    for (int i = 0; ok && i < n; i++)
        ok = A->Len[i] == 0 || fwrite(A->Values[i], sizeof(double), A->Len[i], f) == (size_t)A->Len[i];
    return (fclose(f) == 0 && ok) ? 1 : 0;
}

sparse_matrix* read_sparse(char* path, char* name) {
    if (!path || !name) return nullptr;
    std::string file = std::string(path) + "/" + name;
    lina::Csr c;
    // the file does not say how many columns the matrix has: only negative indices are rejected
    if (!lina::read_csr_file(file, c, INT32_MAX)) return nullptr;
    sparse_matrix* A = (sparse_matrix*)malloc(sizeof(sparse_matrix));
    A->size = c.n;
    A->Len = (int*)malloc(std::max(c.n, 1) * sizeof(int));
    A->Indices = (int**)malloc(std::max(c.n, 1) * sizeof(int*));
    A->Values = (double**)malloc(std::max(c.n, 1) * sizeof(double*));
    for (int i = 0; i < c.n; i++) {
        const int len = c.ptr[i + 1] - c.ptr[i];
        A->Len[i] = len;
        A->Indices[i] = (int*)malloc(std::max(len, 1) * sizeof(int));
        A->Values[i] = (double*)malloc(std::max(len, 1) * sizeof(double));
        std::copy(c.col.begin() + c.ptr[i], c.col.begin() + c.ptr[i + 1], A->Indices[i]);
        std::copy(c.val.begin() + c.ptr[i], c.val.begin() + c.ptr[i + 1], A->Values[i]);
    }
    return A;
}

sparse_matrix* get_transpose(sparse_matrix* A, int new_size) {
    sparse_matrix* R = sparse_zero(new_size);
    for (int i = 0; i < A->size; i++)
        for (int r = 0; r < A->Len[i]; r++) insert_sparse(R, A->Values[i][r], A->Indices[i][r], i);
    return R;
}

void sparse_add(sparse_matrix* A, sparse_matrix* B, double factor) {
    if (!B) return;
    for (int i = 0; i < A->size; i++)
        for (int j = 0; j < B->Len[i]; j++) insert_sparse(A, factor * B->Values[i][j], i, B->Indices[i][j]);
}

// row-wise product with accumulation in the order of A's row entries; zero
// factors skipped; zero results deleted (linear_algebra.c:186-222)
sparse_matrix* sparse_product(sparse_matrix* A, sparse_matrix* B) {
    int n = A->size;
    sparse_matrix* P = sparse_zero(n);
    int width = B->size;
    for (int i = 0; i < B->size; i++)
        for (int k = 0; k < B->Len[i]; k++) width = max(width, B->Indices[i][k] + 1);
    width = max(width, n);
    std::vector<double> acc(width, 0.0);
    std::vector<int> mark(width, -1);
    std::vector<int> cols;
    for (int i = 0; i < n; i++) {
        cols.assign(1, i);
        mark[i] = i;
        acc[i] = 0.0;
        for (int p = 0; p < A->Len[i]; p++) {
            double a = A->Values[i][p];
            if (a == 0) continue;
            int k = A->Indices[i][p];
            for (int q = 0; q < B->Len[k]; q++) {
                double b = B->Values[k][q];
                if (b == 0) continue;
                int j = B->Indices[k][q];
                if (mark[j] != i) {
                    mark[j] = i;
                    acc[j] = a * b;
                    cols.push_back(j);
                } else {
                    acc[j] += a * b;
                }
            }
        }
        std::sort(cols.begin(), cols.end());
        int len = (int)cols.size();
        P->Values[i] = (double*)realloc(P->Values[i], len * sizeof(double));
        P->Indices[i] = (int*)realloc(P->Indices[i], len * sizeof(int));
        for (int k = 0; k < len; k++) {
            P->Indices[i][k] = cols[k];
            P->Values[i][k] = acc[cols[k]];
        }
        P->Len[i] = len;
    }
    delete_zeros(P);
    return P;
}

double* sparse_row_sum(sparse_matrix* A) {
    double* r = zero_vector(A->size);
    for (int i = 0; i < A->size; i++)
        for (int j = 0; j < A->Len[i]; j++) r[i] += A->Values[i][j];
    return r;
}

void scalar_sparse_mult(double a, sparse_matrix* A) {
    for (int i = 0; i < A->size; i++)
        for (int j = 0; j < A->Len[i]; j++) A->Values[i][j] *= a;
}

sparse_matrix* make_positive_diag(sparse_matrix* A) {
    sparse_matrix* S = sparse_identity(A->size);
    for (int i = 0; i < A->size; i++)
        if (get_diag(A, i) < 0) {
            for (int j = 0; j < A->Len[i]; j++) A->Values[i][j] *= -1.;
            S->Values[i][0] *= -1.;
        }
    return S;
}

int diag_zero(sparse_matrix* A) {
    for (int i = 0; i < A->size; i++)
        if (get_diag(A, i) == 0) {
            printf("zero diagonal at index %d\n", i);
            return 1;
        }
    return 0;
}

// five-point Laplacian with identity boundary rows (linear_algebra.c:4312)
sparse_matrix* Lap_2D_Dirichlet(double a, double b, int dom_size) {
    int N = dom_size * dom_size;
    sparse_matrix* A = sparse_zero(N);
    for (int i = 1; i < dom_size - 1; i++)
        for (int j = 1; j < dom_size - 1; j++) {
            int k = i * dom_size + j;
            insert_sparse(A, 2. * (a + b), k, k);
            insert_sparse(A, -a, k, (i + 1) * dom_size + j);
            insert_sparse(A, -a, k, (i - 1) * dom_size + j);
            insert_sparse(A, -b, k, i * dom_size + j + 1);
            insert_sparse(A, -b, k, i * dom_size + j - 1);
        }
    for (int i = 0; i < dom_size; i++) {
        insert_sparse(A, 1., i * dom_size, i * dom_size);
        insert_sparse(A, 1., i * dom_size + dom_size - 1, i * dom_size + dom_size - 1);
        insert_sparse(A, 1., i, i);
        insert_sparse(A, 1., (dom_size - 1) * dom_size + i, (dom_size - 1) * dom_size + i);
    }
    return A;
}

double* sparse_mult(sparse_matrix* A, double* x) {
    double* y = (double*)malloc((A->size > 0 ? A->size : 1) * sizeof(double));
    for (int i = 0; i < A->size; i++) {
        double s = 0;
        for (int j = 0; j < A->Len[i]; j++) s += A->Values[i][j] * x[A->Indices[i][j]];
        y[i] = s;
    }
    return y;
}

void linear_map(double* x, double fac, sparse_matrix* A, double* y) {
    for (int i = 0; i < A->size; i++) {
        double s = 0;
        for (int j = 0; j < A->Len[i]; j++) s += A->Values[i][j] * y[A->Indices[i][j]];
        s *= fac;
        x[i] += s;
    }
}

void sparse_multiplication(sparse_matrix* A, double* x) {
    double* y = sparse_mult(A, x);
    memcpy(x, y, A->size * sizeof(double));
    free(y);
}

double sparse_bilinear(double* y, sparse_matrix* A, double* x) {
    double* Ax = sparse_mult(A, x);
    double r = scalar(y, Ax, A->size);
    free(Ax);
    return r;
}

double matrix_residuum(sparse_matrix* A, double* Sol, double* b) {
    double* R = clone_vector(b, A->size);
    linear_map(R, -1., A, Sol);
    double r = euklid_norm(R, A->size);
    free(R);
    return r;
}

// ILU(0) on A's pattern: L lower with its diagonal, U upper with unit diagonal
// (linear_algebra.c:1952-1982); returns 0 on a zero pivot
static double row_dot(sparse_matrix* A, sparse_matrix* B, int ia, int ib, int jmax) {
    // sum over k <= jmax of A[ia][k] * B[ib][k], rows sorted (row_times_row, :1795)
    double s = 0;
    int p = 0, q = 0;
    while (p < A->Len[ia] && q < B->Len[ib]) {
        int ca = A->Indices[ia][p], cb = B->Indices[ib][q];
        if (ca > jmax) break;
        if (ca == cb) {
            s += A->Values[ia][p] * B->Values[ib][q];
            p++;
            q++;
        } else if (ca < cb) {
            p++;
        } else {
            q++;
        }
    }
    return s;
}

int incomplete_LU_factorization(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U) {
    int n = A->size;
    for (int i = 0; i < n; i++) {
        insert_sparse(U, 1., i, i);
        for (int jr = 0; jr < A->Len[i]; jr++) {
            int j = A->Indices[i][jr];
            double sum = A->Values[i][jr];
            if (j <= i) {
                sum -= row_dot(L, U, i, j, j - 1);
                insert_sparse(L, sum, i, j);
            } else {
                sum -= row_dot(L, U, i, j, i - 1);
                double d = get_matrix_element(L, i, i);
                if (d == 0) return 0;
                sum /= d;
                insert_sparse(U, sum, j, i);
            }
        }
    }
    sparse_matrix* T = get_transpose(U, n);
    for (int i = 0; i < n; i++) {
        free(U->Values[i]);
        free(U->Indices[i]);
        U->Values[i] = T->Values[i];
        U->Indices[i] = T->Indices[i];
        U->Len[i] = T->Len[i];
    }
    free(T->Values);
    free(T->Indices);
    free(T->Len);
    free(T);
    return 1;
}

void L_triang_invert(sparse_matrix* L, double* x) {
    for (int i = 0; i < L->size; i++) {
        double sum = x[i], diag = 0;
        for (int j = 0; j < L->Len[i]; j++) {
            int J = L->Indices[i][j];
            if (J != i)
                sum -= L->Values[i][j] * x[J];
            else
                diag = L->Values[i][j];
        }
        x[i] = sum / diag;
    }
}

void U_triang_invert(sparse_matrix* U, double* x) {
    for (int i = U->size - 1; i >= 0; i--) {
        double sum = x[i], diag = 0;
        for (int j = 0; j < U->Len[i]; j++) {
            int J = U->Indices[i][j];
            if (J != i)
                sum -= U->Values[i][j] * x[J];
            else
                diag = U->Values[i][j];
        }
        x[i] = sum / diag;
    }
}

double ILU_residuum(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U, double* Sol, double* b) {
    double* R = clone_vector(b, A->size);
    linear_map(R, -1., A, Sol);
    L_triang_invert(L, R);
    U_triang_invert(U, R);
    double r = euklid_norm(R, A->size);
    free(R);
    return r;
}

}  // extern "C"

// ============================================================ row list <-> CSR
namespace lina {
namespace api {

CsrCopy to_csr(const sparse_matrix* A) {
    CsrCopy c;
    c.n = A->size;
    c.ptr.assign(c.n + 1, 0);
    for (int i = 0; i < c.n; i++) c.ptr[i + 1] = c.ptr[i] + A->Len[i];
    c.col.resize(c.ptr[c.n]);
    c.val.resize(c.ptr[c.n]);
    for (int i = 0; i < c.n; i++) {
        memcpy(c.col.data() + c.ptr[i], A->Indices[i], A->Len[i] * sizeof(int));
        memcpy(c.val.data() + c.ptr[i], A->Values[i], A->Len[i] * sizeof(double));
    }
    return c;
}

sparse_matrix* from_csr(int n, const int* ptr, const int* col, const double* val) {
    sparse_matrix* A = (sparse_matrix*)malloc(sizeof(sparse_matrix));
    A->size = n;
    A->Len = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
    A->Values = (double**)malloc((n > 0 ? n : 1) * sizeof(double*));
    A->Indices = (int**)malloc((n > 0 ? n : 1) * sizeof(int*));
    for (int i = 0; i < n; i++) {
        int len = ptr[i + 1] - ptr[i];
        int alloc = len > 0 ? len : 1;
        A->Values[i] = (double*)malloc(alloc * sizeof(double));
        A->Indices[i] = (int*)malloc(alloc * sizeof(int));
        if (len == 0) {
            A->Values[i][0] = 0.0;
            A->Indices[i][0] = i;
            A->Len[i] = 1;
        } else {
            memcpy(A->Values[i], val + ptr[i], len * sizeof(double));
            memcpy(A->Indices[i], col + ptr[i], len * sizeof(int));
            A->Len[i] = len;
        }
    }
    return A;
}

// content fingerprint of a row-list matrix (decides whether a device copy is current)
uint64_t fingerprint(const sparse_matrix* A) {
    uint64_t h = 1469598103934665603ull ^ (uint64_t)A->size;
    auto mix = [&](uint64_t v) {
        h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    };
    for (int i = 0; i < A->size; i++) {
        mix((uint64_t)A->Len[i]);
        for (int k = 0; k < A->Len[i]; k++) {
            uint64_t b;
            memcpy(&b, &A->Values[i][k], sizeof b);
            mix(b ^ ((uint64_t)(uint32_t)A->Indices[i][k] << 1));
        }
    }
    return h;
}

}  // namespace api
}  // namespace lina

namespace {
using namespace lina::api;

// device copies of caller matrices used as operators (PCG_mult, BiCGStab products)
struct DevMat {
    lina_gpu_matrix* m = nullptr;
    uint64_t fp = 0;
    int n = 0;
};
std::unordered_map<const sparse_matrix*, DevMat> g_devmats;

}  // namespace

void lina::api::forget_device_matrix(const sparse_matrix* A) {
    auto it = g_devmats.find(A);
    if (it == g_devmats.end()) return;
    if (it->second.m) lina_gpu_matrix_destroy(it->second.m);
    g_devmats.erase(it);
}

lina_gpu_matrix* lina::api::device_matrix(const sparse_matrix* A) {
    uint64_t fp = fingerprint(A);
    DevMat& d = g_devmats[A];
    if (d.m && d.fp == fp && d.n == A->size) return d.m;
    if (d.m) lina_gpu_matrix_destroy(d.m);
    d.m = nullptr;
    CsrCopy c = to_csr(A);
    int ncols = c.n;
    for (int v : c.col) ncols = std::max(ncols, v + 1);
    if (lina_gpu_matrix_create(c.n, ncols, c.ptr.data(), c.col.data(), c.val.data(), &d.m) != 0) {
        fprintf(stderr, "LinA-GB300: device copy of a matrix failed: %s\n", lina_gpu_last_error());
        d.m = nullptr;
        return nullptr;
    }
    d.fp = fp;
    d.n = A->size;
    return d.m;
}

// device ILU(0) of the factors given to PCG_default (PCG_preconlr on the GPU)
namespace {
struct DevIlu {
    lina_gpu_ilu* h = nullptr;
    uint64_t fpl = 0, fpu = 0;
    const sparse_matrix *L = nullptr, *U = nullptr;
} g_devilu;
}  // namespace

lina_gpu_ilu* lina::api::device_ilu(const sparse_matrix* L, const sparse_matrix* U) {
    uint64_t fl = fingerprint(L), fu = fingerprint(U);
    if (g_devilu.h && g_devilu.L == L && g_devilu.U == U && g_devilu.fpl == fl && g_devilu.fpu == fu)
        return g_devilu.h;
    if (g_devilu.h) lina_gpu_ilu_destroy(g_devilu.h);
    g_devilu = DevIlu();
    CsrCopy l = to_csr(L), u = to_csr(U);
    if (lina_gpu_ilu_create(l.n, l.ptr.data(), l.col.data(), l.val.data(), u.ptr.data(), u.col.data(), u.val.data(),
                            &g_devilu.h) != 0) {
        fprintf(stderr, "LinA-GB300: device ILU factors could not be created\n");
        g_devilu.h = nullptr;
        return nullptr;
    }
    g_devilu.L = L;
    g_devilu.U = U;
    g_devilu.fpl = fl;
    g_devilu.fpu = fu;
    return g_devilu.h;
}

namespace {

// host staging buffers for callbacks
struct Stage {
    std::vector<double> a, b;
    void ensure(int n) {
        if ((int)a.size() < n) {
            a.resize(n);
            b.resize(n);
        }
    }
} g_stage;

}  // namespace

// ============================================================ AMG (Multigrid.c)
namespace {

double amg_eps_minus = 0.3, amg_eps_plus = 0.5, amg_tol = 1.0e-1;  // Multigrid.c:35-37
int amg_max_iter = 20;                                              // :41
double amg_eps = 1e-8;                                              // :42
double sor_alpha = 1.;                                              // :45
int amg_info = YES;                                                 // :49
int amg_dof = 1;                                                    // :50
int gpu_precision = LINA_PREC_FP64;
void (*amg_smoother)(sparse_matrix*, double*, double*, int*, double, int, int, int) = nullptr;

std::unordered_map<amg_system_info*, lina_gpu_amg*> g_amg;
// the caller's matrix each hierarchy was built from (AMG_setup, AMG_recompute_coarse_matrices)
std::unordered_map<amg_system_info*, const sparse_matrix*> g_amg_source;

// the GPU smoother standing for the installed smoother function
bool gpu_smoother(int* kind, double* omega) {
    if (amg_smoother == nullptr || amg_smoother == AMG_SOR_smoother) {
        *kind = LINA_SMOOTHER_MC_SOR;
        *omega = sor_alpha;
        return true;
    }
    if (amg_smoother == AMG_parallel_Jacobi_smoother) {
        *kind = LINA_SMOOTHER_JACOBI;
        *omega = 1.0;
        return true;
    }
    if (amg_smoother == AMG_damped_Jacobi_smoother) {
        *kind = LINA_SMOOTHER_JACOBI;
        *omega = sor_alpha;
        return true;
    }
    return false;
}

int* default_iterations(int depth) {
    int* it = (int*)malloc(depth * sizeof(int));
    for (int i = 0; i < depth; i++) it[i] = 1;
    return it;
}

void fill_info_levels(amg_system_info* I, lina_gpu_amg* h) {
    const int depth = I->depth;
    for (int l = 0; l < depth; l++) {
        int n = 0, nc = 0;
        long na = 0, np = 0, nr = 0;
        lina_gpu_level_sizes(h, l, &n, &na, &np, &nr, &nc);
        std::vector<int> lab(n), ap(n + 1), ac(na > 0 ? na : 1);
        std::vector<double> av(na > 0 ? na : 1);
        int ncoarse = 0;
        if (l > 0) lina_gpu_level_sizes(h, l - 1, &ncoarse, nullptr, nullptr, nullptr, nullptr);
        std::vector<int> pp(n + 1), pc(np > 0 ? np : 1), rp(ncoarse + 1), rc(nr > 0 ? nr : 1);
        std::vector<double> pv(np > 0 ? np : 1), rv(nr > 0 ? nr : 1);
        lina_gpu_level_export(h, l, lab.data(), ap.data(), ac.data(), av.data(), l > 0 ? pp.data() : nullptr,
                              l > 0 ? pc.data() : nullptr, l > 0 ? pv.data() : nullptr, l > 0 ? rp.data() : nullptr,
                              l > 0 ? rc.data() : nullptr, l > 0 ? rv.data() : nullptr);
        I->Coarse_A[l] = from_csr(n, ap.data(), ac.data(), av.data());
        I->Fine_sizes[l] = n;
        I->L[l] = nullptr;
        I->U[l] = nullptr;
        if (l > 0) {
            I->Coarse_sizes[l] = ncoarse;
            I->Prolongation[l] = from_csr(n, pp.data(), pc.data(), pv.data());
            I->Restriction[l] = from_csr(ncoarse, rp.data(), rc.data(), rv.data());
            I->Coarsening[l] = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
            memcpy(I->Coarsening[l], lab.data(), n * sizeof(int));
        } else {
            I->Coarse_sizes[l] = 0;
            I->Prolongation[l] = nullptr;
            I->Restriction[l] = nullptr;
            I->Coarsening[l] = nullptr;
        }
    }
}

void free_info_levels(amg_system_info* I) {
    for (int i = 0; i < I->depth; i++) {
        if (I->Coarse_A[i]) { free_sparse(I->Coarse_A[i]); }
        if (I->Prolongation[i]) { free_sparse(I->Prolongation[i]); }
        if (I->Restriction[i]) { free_sparse(I->Restriction[i]); }
        if (I->L[i]) { free_sparse(I->L[i]); }
        if (I->U[i]) { free_sparse(I->U[i]); }
        if (I->Coarsening[i]) free(I->Coarsening[i]);
        I->Coarse_A[i] = I->Prolongation[i] = I->Restriction[i] = I->L[i] = I->U[i] = nullptr;
        I->Coarsening[i] = nullptr;
    }
}

}  // namespace

extern "C" {

void AMG_set_SOR_relaxation_coeff(double alpha) { sor_alpha = alpha; }
void set_connection_thresholds(double negative, double positive) {
    amg_eps_minus = negative;
    amg_eps_plus = positive;
}
void AMG_set_eps(double eps) { amg_eps = eps; }
void AMG_set_max_iter(int iter) { amg_max_iter = iter; }
int AMG_get_max_iter(void) { return amg_max_iter; }
void AMG_set_deg_of_freedom(int n) { amg_dof = n; }
void AMG_set_matrix_tolerance(double tol) { amg_tol = tol; }
void AMG_set_smoother(void (*Smoother)(sparse_matrix*, double*, double*, int*, double, int, int, int)) {
    amg_smoother = Smoother;
}
void AMG_print_info(int s) { amg_info = s; }
int AMG_info_set(void) { return amg_info; }
void AMG_gpu_set_precision(int precision) { gpu_precision = precision ? LINA_PREC_MIXED : LINA_PREC_FP64; }
int* AMG_default_iterations(int depth) { return default_iterations(depth); }

// The smoothers keep their reference meaning when called directly on a host
// system (Multigrid.c:1345-1400); as arguments of AMG_set_smoother they select
// the GPU smoother of AMG_solve (multicolour SOR, Jacobi, damped Jacobi).
void AMG_SOR_smoother(sparse_matrix* A, double* F, double* Sol, int* Label, double alpha, int fix, int iter,
                      int deg_freedom) {
    (void)deg_freedom;
    for (int k = 0; k < iter; k++)
        for (int i = 0; i < A->size; i++) {
            if (Label && Label[i] == fix) continue;
            double sum = F[i];
            int diag = -1;
            for (int j = 0; j < A->Len[i]; j++) {
                int ind = A->Indices[i][j];
                if (ind != i)
                    sum -= A->Values[i][j] * Sol[ind];
                else
                    diag = j;
            }
            if (diag < 0) {
                printf("diagonal element is zero at index %d -> abort SOR\n", i);
                return;
            }
            Sol[i] = (1. - alpha) * Sol[i] + alpha * sum / A->Values[i][diag];
        }
}

static void jacobi_host(sparse_matrix* A, double* F, double* Sol, int* Label, double w, int fix, int iter) {
    std::vector<double> old(A->size);
    for (int k = 0; k < iter; k++) {
        memcpy(old.data(), Sol, A->size * sizeof(double));
        for (int i = 0; i < A->size; i++) {
            if (Label && Label[i] == fix) continue;
            double sum = F[i], aii = 0;
            for (int j = 0; j < A->Len[i]; j++) {
                int ind = A->Indices[i][j];
                if (ind != i)
                    sum -= A->Values[i][j] * old[ind];
                else
                    aii = A->Values[i][j];
            }
            Sol[i] = (1. - w) * old[i] + w * sum / aii;
        }
    }
}

void AMG_parallel_Jacobi_smoother(sparse_matrix* A, double* F, double* Sol, int* Label, double alpha, int fix,
                                  int iter, int deg_freedom) {
    (void)alpha;
    (void)deg_freedom;
    jacobi_host(A, F, Sol, Label, 1.0, fix, iter);
}

void AMG_damped_Jacobi_smoother(sparse_matrix* A, double* F, double* Sol, int* Label, double alpha, int fix,
                                int iter, int deg_freedom) {
    (void)deg_freedom;
    jacobi_host(A, F, Sol, Label, alpha, fix, iter);
}

amg_system_info* AMG_setup(sparse_matrix* A, int deg_of_freedom, int depth, int smoothing_iterations,
                           int aggr_smoothing_iterations, int coarsening, int cycle_structure,
                           int prolongation_method,
                           void (*coarsest_solver)(sparse_matrix*, sparse_matrix*, double*, double*, int),
                           int* (*Get_iter)(int depth)) {
    (void)prolongation_method;
    if (cycle_structure != STAND_ALONE && cycle_structure != FULL_AMG)
        fprintf(stderr, "LinA-GB300: unknown cycle structure %d; AMG_solve will skip the solution\n", cycle_structure);
    if (coarsest_solver != nullptr)
        fprintf(stderr, "LinA-GB300: a custom coarsest-level solver is not used; the GPU solves the coarsest level\n");
    if (Get_iter != nullptr && Get_iter != AMG_default_iterations)
        fprintf(stderr, "LinA-GB300: custom cycle counts are not used; one cycle per level\n");
    amg_dof = deg_of_freedom;
    CsrCopy c = to_csr(A);
    lina_gpu_amg_options o;
    lina_gpu_default_options(&o);
    o.dof = deg_of_freedom;
    o.depth = depth;
    o.smoothing_iterations = smoothing_iterations;
    o.aggr_smoothing_iterations = aggr_smoothing_iterations;
    o.coarsening = (coarsening == AGGRESSIVE) ? LINA_AGGRESSIVE : (coarsening == LINA_PMIS) ? LINA_PMIS : LINA_STANDARD;
    o.eps_minus = amg_eps_minus;
    o.eps_plus = amg_eps_plus;
    o.matrix_tol = amg_tol;
    int kind;
    double omega;
    if (!gpu_smoother(&kind, &omega)) {
        kind = LINA_SMOOTHER_MC_SOR;
        omega = sor_alpha;
    }
    o.smoother = kind;
    o.omega = omega;
    o.precision = gpu_precision;
    lina_gpu_amg* h = nullptr;
    if (lina_gpu_amg_create(c.n, c.ptr.data(), c.col.data(), c.val.data(), &o, &h) != 0) {
        fprintf(stderr, "LinA-GB300: AMG_setup failed: %s\n", lina_gpu_last_error());
        return nullptr;
    }
    amg_system_info* I = (amg_system_info*)calloc(1, sizeof(amg_system_info));
    I->depth = depth;
    I->Coarse_A = (sparse_matrix**)calloc(depth, sizeof(sparse_matrix*));
    I->Prolongation = (sparse_matrix**)calloc(depth, sizeof(sparse_matrix*));
    I->Restriction = (sparse_matrix**)calloc(depth, sizeof(sparse_matrix*));
    I->L = (sparse_matrix**)calloc(depth, sizeof(sparse_matrix*));
    I->U = (sparse_matrix**)calloc(depth, sizeof(sparse_matrix*));
    I->Coarsening = (int**)calloc(depth, sizeof(int*));
    I->Coarse_sizes = (int*)calloc(depth, sizeof(int));
    I->Fine_sizes = (int*)calloc(depth, sizeof(int));
    I->AMG_deg_of_freedom = deg_of_freedom;
    I->AMG_smoothing_iterations = smoothing_iterations;
    I->AMG_aggr_smoothing_iterations = aggr_smoothing_iterations;
    I->AMG_coarsening = coarsening;
    I->AMG_cycle_structure = cycle_structure;
    I->AMG_prolongation_method = prolongation_method;
    I->AMG_info = amg_info;
    I->Get_iter = AMG_default_iterations;
    fill_info_levels(I, h);
    // signs of make_positive_diag
    sparse_matrix* S = sparse_identity(A->size);
    for (int i = 0; i < A->size; i++)
        if (get_diag(A, i) < 0) S->Values[i][0] = -1.;
    I->Signs = S;
    g_amg[I] = h;
    g_amg_source[I] = A;
    return I;
}

int AMG_solve(amg_system_info* Data, double* F, double* Fine_Sol, amg_statistics* Stat) {
    auto it = g_amg.find(Data);
    if (it == g_amg.end()) {
        fprintf(stderr, "LinA-GB300: AMG_solve on data that AMG_setup did not create\n");
        return -1;
    }
    lina_gpu_amg* h = it->second;
    int kind;
    double omega;
    if (!gpu_smoother(&kind, &omega)) {
        fprintf(stderr, "LinA-GB300: AMG_solve: a caller-defined smoother cannot run in the GPU V-cycle\n");
        return -1;
    }
    lina_gpu_amg_set_smoother(h, kind, omega, gpu_precision);
    int iters = 0;
    double rel = 0;
    if (Data->AMG_cycle_structure == FULL_AMG) {
        // one full-multigrid pass (Multigrid.c:1908-1911); the reference's statistics keep r/r0 = 1
        // because it does not recompute r after the pass
        double r = 0;
        int rc = lina_gpu_amg_fmg(h, F, Fine_Sol, 0, &r);
        if (rc != 0 && rc != LINA_GPU_EBREAKDOWN) {
            fprintf(stderr, "LinA-GB300: AMG_solve failed: %s\n", lina_gpu_last_error());
            return -1;
        }
        if (Stat) AMG_add_stat(Stat, 1, r == 0 ? 0.0 : 1.0);
        if (amg_info == YES) {
            printf("\niterations: %d\n", 1);
            printf("total relative residuum: %e\n", 1.0);
        }
        return 1;
    }
    if (Data->AMG_cycle_structure != STAND_ALONE) {
        printf("Warning AMG: no solution method choosen -> skip\n");
        return 0;
    }
    int rc = lina_gpu_amg_solve(h, F, Fine_Sol, amg_eps, amg_max_iter, 0, &iters, &rel);
    if (rc != 0 && rc != LINA_GPU_EBREAKDOWN) {
        fprintf(stderr, "LinA-GB300: AMG_solve failed: %s\n", lina_gpu_last_error());
        return -1;
    }
    if (Stat) AMG_add_stat(Stat, iters, fabs(rel));
    if (amg_info == YES) {
        printf("\niterations: %d\n", iters);
        printf("total relative residuum: %e\n", rel);
    }
    return iters;
}

void AMG_recompute_coarse_matrices(amg_system_info* Info, sparse_matrix* New_matrix) {
    auto it = g_amg.find(Info);
    if (it == g_amg.end()) return;
    CsrCopy c = to_csr(New_matrix);
    if (lina_gpu_amg_recompute(it->second, c.n, c.ptr.data(), c.col.data(), c.val.data()) != 0) {
        fprintf(stderr, "LinA-GB300: AMG_recompute_coarse_matrices failed: %s\n", lina_gpu_last_error());
        return;
    }
    free_info_levels(Info);
    fill_info_levels(Info, it->second);
    g_amg_source[Info] = New_matrix;
}

void AMG_free_data(amg_system_info* Data) {
    auto it = g_amg.find(Data);
    if (it != g_amg.end()) {
        lina_gpu_amg_destroy(it->second);
        g_amg.erase(it);
    }
    g_amg_source.erase(Data);
    free_info_levels(Data);
    if (Data->Signs) { free_sparse(Data->Signs); }
    free(Data->Coarse_A);
    free(Data->Prolongation);
    free(Data->Restriction);
    free(Data->L);
    free(Data->U);
    free(Data->Coarsening);
    free(Data->Fine_sizes);
    free(Data->Coarse_sizes);
}

amg_statistics AMG_init_stat(const char* Out) {
    amg_statistics s;
    s.calls = 0;
    s.Iterations = nullptr;
    s.Residuals = nullptr;
    s.max_iter = 0;
    s.max_res = 0;
    snprintf(s.File_name, sizeof s.File_name, "%s", Out ? Out : "");
    return s;
}

void AMG_add_stat(amg_statistics* Stat, int iter, double res) {
    int i = Stat->calls++;
    Stat->Iterations = (int*)realloc(Stat->Iterations, Stat->calls * sizeof(int));
    Stat->Residuals = (double*)realloc(Stat->Residuals, Stat->calls * sizeof(double));
    Stat->Iterations[i] = iter;
    Stat->Residuals[i] = res;
    if (res > Stat->max_res) Stat->max_res = res;
    if (iter > Stat->max_iter) Stat->max_iter = iter;
}

void AMG_print_stat(amg_statistics* Stat) {
    printf("\nstatistics output: %s\n", Stat->File_name);
    printf("calls: %d\n", Stat->calls);
    int isum = 0;
    double dsum = 0;
    for (int i = 0; i < Stat->calls; i++) {
        isum += Stat->Iterations[i];
        dsum += Stat->Residuals[i];
    }
    printf("average iterations: %f\n", Stat->calls ? (float)isum / Stat->calls : 0.f);
    printf("average residual: %e\n", Stat->calls ? (float)dsum / Stat->calls : 0.f);
    printf("maximum iterations: %d\n", Stat->max_iter);
    printf("maximum residual: %e\n\n", Stat->max_res);
}

}  // extern "C"

// ============================================================ operators on device vectors
namespace {

using MatMult = void (*)(int, double*, double*);
using Precon = int (*)(int, double*, double*);

sparse_matrix* pcg_default_A = nullptr;
sparse_matrix* pcg_default_L = nullptr;
sparse_matrix* pcg_default_U = nullptr;
amg_system_info* pcg_amg_data = nullptr;
amg_system_info* bi_amg_data = nullptr;
amg_statistics bi_amg_stat;
amg_statistics bi_stat;

// y = A x on device vectors: the library's own product runs on the GPU, a
// caller's callback runs on host copies
bool apply_matmult(MatMult f, sparse_matrix* own, int n, const double* x, double* y) {
    if (f == RN_default_mat_mult) own = lina::api::rn_default_matrix();
    if ((f == PCG_mult || f == RN_default_mat_mult) && own) {
        lina_gpu_matrix* m = device_matrix(own);
        if (!m) return false;
        lina::dev::sync();
        return lina_gpu_matrix_spmv(m, LINA_PREC_FP64, x, y) == 0;
    }
    g_stage.ensure(n);
    if (!lina::dev::d2h(g_stage.a.data(), x, n)) return false;
    f(n, g_stage.a.data(), g_stage.b.data());
    return lina::dev::h2d(y, g_stage.b.data(), n);
}

// Z = M^-1 R; the AMG preconditioners warm-start from the incoming Z like
// AMG_solve does on the host (PCGS.c:114, BiCGStab.c:84)
int apply_precon(Precon f, int n, const double* r, double* z, amg_statistics* stat) {
    if (f == PCG_AMG_vcycle_precon) {
        auto it = g_amg.find(pcg_amg_data);
        int kind;
        double omega;
        if (it == g_amg.end() || !gpu_smoother(&kind, &omega)) return -1;
        lina_gpu_amg_set_smoother(it->second, kind, omega, gpu_precision);
        if (!lina::dev::zero(z, n)) return -1;
        lina::dev::sync();
        int iters = 0;
        double rel = 0;
        int rc = lina_gpu_amg_solve(it->second, r, z, 0.0, 1, LINA_PCG_DEVICE_PTRS, &iters, &rel);
        return (rc != 0 && rc != LINA_GPU_EBREAKDOWN) ? -1 : iters;
    }
    amg_system_info* data = nullptr;
    if (f == PCG_AMG_precon) data = pcg_amg_data;
    if (f == BI_AMG_precon) data = bi_amg_data;
    if (data) {
        auto it = g_amg.find(data);
        if (it == g_amg.end()) return -1;
        int kind;
        double omega;
        if (!gpu_smoother(&kind, &omega)) {
            fprintf(stderr, "LinA-GB300: a caller-defined smoother cannot run in the GPU V-cycle\n");
            return -1;
        }
        lina_gpu_amg_set_smoother(it->second, kind, omega, gpu_precision);
        lina::dev::sync();
        int iters = 0;
        double rel = 0;
        int rc = lina_gpu_amg_solve(it->second, r, z, amg_eps, amg_max_iter, LINA_PCG_DEVICE_PTRS, &iters, &rel);
        if (rc != 0 && rc != LINA_GPU_EBREAKDOWN) return -1;
        if (stat) AMG_add_stat(stat, iters, fabs(rel));
        return iters;
    }
    if (f == PCG_preconlr) {
        if (!pcg_default_L || !pcg_default_U) return lina::dev::d2d(z, r, n) ? 1 : -1;
        lina_gpu_ilu* ilu = device_ilu(pcg_default_L, pcg_default_U);
        if (!ilu) return -1;
        lina::dev::sync();
        return lina_gpu_ilu_apply(ilu, LINA_PREC_FP64, r, z) == 0 ? 1 : -1;
    }
    g_stage.ensure(n);
    if (!lina::dev::d2h(g_stage.a.data(), r, n) || !lina::dev::d2h(g_stage.b.data(), z, n)) return -1;
    int k = f(n, g_stage.a.data(), g_stage.b.data());
    if (!lina::dev::h2d(z, g_stage.b.data(), n)) return -1;
    return k;
}

MatMult pcg_mat_multi = nullptr;
Precon pcg_precon = nullptr;
double pcg_res = 0;

}  // namespace

bool lina::api::device_matmult(MatMultFn f, int n, const double* x, double* y) {
    return apply_matmult(f, f == PCG_mult ? pcg_default_A : nullptr, n, x, y);
}

int lina::api::device_precon(PreconFn f, int n, const double* r, double* z) { return apply_precon(f, n, r, z, nullptr); }

namespace {

MatMult bi_mat_mult = nullptr;
Precon bi_precon = nullptr;
int bi_max_iter = 1000;  // BiCGStab.c:12
double bi_eps = 1e-8;    // :13
int bi_info = YES;       // :14

// Work vectors of the drop-in Krylov loops, kept between calls (grown when a larger system comes) so
// that a caller solving repeatedly does not pay device allocations on every call.
struct DevVecs {
    std::vector<double*> v;
    DevVecs(int count, int n) {
        static std::vector<double*> cache;
        static int cache_n = 0;
        if (n > cache_n) {
            for (auto p : cache) lina::dev::release(p);
            cache.clear();
            cache_n = n;
        }
        while ((int)cache.size() < count) cache.push_back(lina::dev::alloc(cache_n));
        v.assign(cache.begin(), cache.begin() + count);
    }
    bool ok() const {
        for (auto p : v)
            if (!p) return false;
        return true;
    }
};

}  // namespace

extern "C" {

void PCG_set_precon(int (*Precon_)(int n, double* R, double* Z)) { pcg_precon = Precon_; }
void PCG_set_mat_mult(void (*Mat_mult)(int n, double* x, double* y)) { pcg_mat_multi = Mat_mult; }
void* PCG_get_precon(void) { return (void*)pcg_precon; }
void* PCG_get_mat_mult(void) { return (void*)pcg_mat_multi; }
double get_pcg_residuum(void) { return pcg_res; }

void PCG_default(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U) {
    pcg_default_A = A;
    pcg_default_L = L;
    pcg_default_U = U;
    PCG_set_default_precon();
}

void PCG_set_default_precon(void) {
    PCG_set_mat_mult(PCG_mult);
    PCG_set_precon(PCG_preconlr);
}

// z = default_A y, for callers that use the operator directly (PCGS.c:36)
void PCG_mult(int n, double* y, double* z) {
    if (!pcg_default_A) return;
    lina_gpu_matrix* m = device_matrix(pcg_default_A);
    double* dy = lina::dev::alloc(n);
    double* dz = lina::dev::alloc(n);
    if (m && dy && dz && lina::dev::h2d(dy, y, n) && lina_gpu_matrix_spmv(m, LINA_PREC_FP64, dy, dz) == 0)
        lina::dev::d2h(z, dz, n);
    lina::dev::release(dy);
    lina::dev::release(dz);
}

// w = U^-1 L^-1 z with the factors given to PCG_default (PCGS.c:61-108)
int PCG_preconlr(int n, double* z, double* w) {
    if (!pcg_default_L || !pcg_default_U) {
        copy_vector_to(z, w, n);
        return 1;
    }
    lina_gpu_ilu* ilu = device_ilu(pcg_default_L, pcg_default_U);
    double* dz = lina::dev::alloc(n);
    double* dw = lina::dev::alloc(n);
    int ok = ilu && dz && dw && lina::dev::h2d(dz, z, n) && lina_gpu_ilu_apply(ilu, LINA_PREC_FP64, dz, dw) == 0 &&
             lina::dev::d2h(w, dw, n);
    lina::dev::release(dz);
    lina::dev::release(dw);
    return ok ? 1 : 0;
}

int PCG_AMG_precon(int n, double* Y, double* X) {
    (void)n;
    return AMG_solve(pcg_amg_data, Y, X, nullptr);
}

// One V-cycle of the hierarchy set by PCG_set_AMG_data (or PCG_set_AMG_preconditioner) from the zero
// guess: Z = M^-1 R with the isolated-row fix.  No counterpart in the reference (whose PCG_AMG_precon
// warm-starts AMG_solve from the incoming Z and repeats V-cycles to AMG_eps); installed with
// PCG_set_precon it makes pcg run entirely on the device (see pcg).
int PCG_AMG_vcycle_precon(int n, double* R, double* Z) {
    auto it = g_amg.find(pcg_amg_data);
    if (it == g_amg.end()) {
        fprintf(stderr, "LinA-GB300: PCG_AMG_vcycle_precon without AMG data (PCG_set_AMG_data)\n");
        return -1;
    }
    for (int i = 0; i < n; i++) Z[i] = 0.0;
    const int save_it = amg_max_iter;
    const double save_eps = amg_eps;
    amg_max_iter = 1;
    amg_eps = 0.0;
    const int k = AMG_solve(pcg_amg_data, R, Z, nullptr);
    amg_max_iter = save_it;
    amg_eps = save_eps;
    return k;
}

void PCG_set_AMG_data(amg_system_info* data) { pcg_amg_data = data; }

void PCG_set_AMG_preconditioner(sparse_matrix* A, int num_fields, int depth) {
    AMG_print_info(NO);
    AMG_set_SOR_relaxation_coeff(1.6);
    AMG_set_eps(1e-2);
    AMG_set_max_iter(100);
    printf("set AMG preconditioner: setup ...\n");
    pcg_amg_data = AMG_setup(A, num_fields, depth, 2, 3, AGGRESSIVE, STAND_ALONE, DIRECT, nullptr, nullptr);
    PCG_set_precon(PCG_AMG_precon);
}

namespace {
// pcg with the library's operator and the zero-guess V-cycle: the whole loop on the device as the
// captured graph of lina_gpu_pcg, with the reference's stopping rule ||R|| / ||M^-1 R_0||, B and X scaled
// by 1/||B|| during the solve, X the initial guess, and the closing preconditioner application that
// gives get_pcg_residuum.  -2 when the fast path does not apply.
int pcg_on_device(double* X, double* B, int n, double tol, int max_iter) {
    if (pcg_precon != PCG_AMG_vcycle_precon || pcg_mat_multi != PCG_mult || !pcg_default_A) return -2;
    auto it = g_amg.find(pcg_amg_data);
    auto src = g_amg_source.find(pcg_amg_data);
    if (it == g_amg.end() || src == g_amg_source.end() || src->second != pcg_default_A || pcg_default_A->size != n)
        return -2;
    int kind;
    double omega;
    if (!gpu_smoother(&kind, &omega)) return -2;
    lina_gpu_amg_set_smoother(it->second, kind, omega, gpu_precision);
    lina_gpu_solve_info info;
    const int rc = lina_gpu_pcg(it->second, B, X, tol, max_iter < 1 ? 1 : max_iter, LINA_STOP_REFERENCE,
                                LINA_PCG_USE_X0 | LINA_PCG_NORMALIZE | LINA_PCG_FINAL_PRECON, &info);
    if (rc == LINA_GPU_EBREAKDOWN || std::isnan(info.pcg_residuum)) {
        printf("Fehler bei PCG: nan -> Abbruch\n");
        pcg_res = info.pcg_residuum;
        return -1;
    }
    if (rc != 0 && rc != LINA_GPU_ENOCONV) {
        fprintf(stderr, "LinA-GB300: pcg failed: %s\n", lina_gpu_last_error());
        return -1;
    }
    if (info.iterations >= max_iter) printf("Warnung: maximale Anzahl von %d Iterationen erreicht\n", info.iterations);
    pcg_res = info.pcg_residuum;
    return info.iterations;
}
}  // namespace

// pcg (PCGS.c:163-233) with every vector on the GPU
int pcg(double* X, double* B, int n, double tol, int max_iter) {
    const int fast = pcg_on_device(X, B, n, tol, max_iter);
    if (fast != -2) return fast;
    DevVecs d(7, n);
    if (!d.ok()) {
        fprintf(stderr, "LinA-GB300: pcg: device allocation failed\n");
        return -1;
    }
    double *x = d.v[0], *b = d.v[1], *R = d.v[2], *W = d.v[3], *Q = d.v[4], *Z = d.v[5], *P = d.v[6];
    if (!lina::dev::h2d(b, B, n) || !lina::dev::h2d(x, X, n)) return -1;
    double h = sqrt(lina::dev::dot(b, b, n));
    if (h == 0) h = 1;
    lina::dev::scal(b, 1.0 / h, n);
    lina::dev::scal(x, 1.0 / h, n);
    lina::dev::zero(W, n);
    lina::dev::zero(Q, n);
    lina::dev::zero(Z, n);
    lina::dev::d2d(R, b, n);
    sparse_matrix* own = pcg_default_A;
    if (!apply_matmult(pcg_mat_multi, own, n, x, Q)) return -1;
    lina::dev::axpy(R, -1., Q, n);
    if (apply_precon(pcg_precon, n, R, W, nullptr) < 0) return -1;
    double r0 = sqrt(lina::dev::dot(W, W, n));
    if (r0 == 0) {
        lina::dev::scal(x, h, n);
        lina::dev::d2h(X, x, n);
        return 0;
    }
    double s = 0, s_old, r;
    int i = 0;
    do {
        if (apply_precon(pcg_precon, n, R, Z, nullptr) < 0) return -1;
        s_old = s;
        s = lina::dev::dot(R, Z, n);
        if (i > 0)
            lina::dev::xpay(P, Z, s / s_old, n);
        else
            lina::dev::d2d(P, Z, n);
        if (!apply_matmult(pcg_mat_multi, own, n, P, Q)) return -1;
        double a = s / lina::dev::dot(P, Q, n);
        lina::dev::axpy(x, a, P, n);
        lina::dev::axpy(R, -a, Q, n);
        r = sqrt(lina::dev::dot(R, R, n));
        i++;
    } while (r / r0 > tol && i < max_iter);
    if (i == max_iter) printf("Warnung: maximale Anzahl von %d Iterationen erreicht\n", i);
    if (apply_precon(pcg_precon, n, R, W, nullptr) < 0) return -1;
    r = sqrt(lina::dev::dot(W, W, n));
    if (std::isnan(r / r0)) {
        // the reference exits the process here (PCGS.c:220-223); the library reports it instead
        printf("Fehler bei PCG: nan -> Abbruch\n");
        pcg_res = r / r0;
        return -1;
    }
    lina::dev::scal(x, h, n);
    if (!lina::dev::d2h(X, x, n)) return -1;
    pcg_res = r / r0;
    return i;
}

// ------------------------------------------------------------ BiCGStab (BiCGStab.c)
void BI_set_precon(int (*Preconditioner)(int n, double* Y, double* X)) { bi_precon = Preconditioner; }
void BI_set_mat_mult(void (*Matrix_multiplication)(int n, double* Y, double* X)) { bi_mat_mult = Matrix_multiplication; }
amg_system_info* BI_get_AMG_setup_data(void) { return bi_amg_data; }
void BI_set_AMG_setup_data(amg_system_info* AMG_data) { bi_amg_data = AMG_data; }
void BI_set_eps(double eps) { bi_eps = eps; }
}  // extern "C"
double lina::api::bi_eps_value() { return bi_eps; }
extern "C" {
void BI_set_max_iter(int max_iter) { bi_max_iter = max_iter; }
int BI_get_max_iter(void) { return bi_max_iter; }
void BI_set_stat(char* Out_AMG, char* Out_BiCGStab) {
    bi_amg_stat = AMG_init_stat(Out_AMG);
    bi_stat = AMG_init_stat(Out_BiCGStab);
}
amg_statistics* BI_get_AMG_stat(void) { return &bi_amg_stat; }
amg_statistics* BI_get_stat(void) { return &bi_stat; }
void BI_print_info(int mode) { bi_info = mode; }
int BI_info_set(void) { return bi_info; }

double BI_residuum(double* X, double* b, int n) {
    double* Res = zero_vector(n);
    bi_mat_mult(n, X, Res);
    vector_add(Res, b, -1., n);
    scalar_mult(-1, Res, n);
    double r = euklid_norm(Res, n);
    free(Res);
    return r;
}

static int BI_PCG_precon(int n, double* Y, double* X) {
    int i = pcg(X, Y, n, 1e-2, 1000);
    if (i == 1000) printf("warning PCG preconditioner could not solve to required residuum reduction\n");
    return i;
}

int BI_AMG_precon(int n, double* Y, double* X) {
    (void)n;
    return AMG_solve(bi_amg_data, Y, X, &bi_amg_stat);
}

void BI_set_PCG_preconditioner(sparse_matrix* A) {
    int n = A->size;
    sparse_matrix* L = sparse_zero(n);
    sparse_matrix* U = sparse_zero(n);
    incomplete_LU_factorization(A, L, U);
    PCG_default(A, L, U);
    PCG_set_default_precon();
    BI_set_precon(BI_PCG_precon);
}

void BI_set_AMG_preconditioner(sparse_matrix* A, int num_fields, int depth) {
    AMG_print_info(NO);
    AMG_set_matrix_tolerance(1e-1);
    AMG_set_max_iter(20);
    AMG_set_eps(1e-4);
    printf("set AMG preconditioner: setup ...\n");
    bi_amg_data = AMG_setup(A, num_fields, depth, 2, 3, AGGRESSIVE, STAND_ALONE, DIRECT, nullptr, nullptr);
    BI_set_precon(BI_AMG_precon);
    printf("finished\n\n");
}

// BiCGStab_solve (BiCGStab.c:115-198) with every vector on the GPU
int BiCGStab_solve(double* X, double* b, int n) {
    const double default_eps = 1e-10;
    DevVecs d(10, n);
    if (!d.ok()) {
        fprintf(stderr, "LinA-GB300: BiCGStab: device allocation failed\n");
        return -1;
    }
    double *x = d.v[0], *bb = d.v[1], *S = d.v[2], *PS = d.v[3], *PP = d.v[4], *APP = d.v[5], *APS = d.v[6],
           *R = d.v[7], *R0 = d.v[8], *P = d.v[9];
    if (!lina::dev::h2d(bb, b, n) || !lina::dev::h2d(x, X, n)) return -1;
    for (double* v : {S, PS, PP, APP, APS}) lina::dev::zero(v, n);
    sparse_matrix* own = pcg_default_A;
    if (!apply_matmult(bi_mat_mult, own, n, x, R)) return -1;
    lina::dev::axpy(R, -1., bb, n);
    lina::dev::scal(R, -1., n);
    lina::dev::d2d(R0, R, n);
    lina::dev::d2d(P, R, n);
    int iter = 0;
    double r0 = sqrt(lina::dev::dot(R, R, n)), r = r0;
    if (r0 == 0 && bi_info == BI_YES) {
        printf("initial residuum zero -> continue ...\n");
    } else {
        do {
            if (apply_precon(bi_precon, n, P, PP, (bi_precon == BI_AMG_precon) ? &bi_amg_stat : nullptr) < 0) return -1;
            if (!apply_matmult(bi_mat_mult, own, n, PP, APP)) return -1;
            double h = lina::dev::dot(R, R0, n);
            double t = lina::dev::dot(APP, R0, n);
            if (t == 0) {
                if (fabs(r0) > default_eps) printf("Warning: BiCGStab stopped because alpha->infinity\n");
                break;
            }
            double alpha = h / t;
            lina::dev::d2d(S, R, n);
            lina::dev::axpy(S, -alpha, APP, n);
            if (apply_precon(bi_precon, n, S, PS, (bi_precon == BI_AMG_precon) ? &bi_amg_stat : nullptr) < 0) return -1;
            if (!apply_matmult(bi_mat_mult, own, n, PS, APS)) return -1;
            double s = lina::dev::dot(APS, APS, n);
            if (s == 0) {
                if (fabs(r0) > default_eps) printf("Warning: BiCGStab stopped because APS=0\n");
                break;
            }
            double omega = lina::dev::dot(APS, S, n) / s;
            lina::dev::axpy(x, alpha, PP, n);
            lina::dev::axpy(x, omega, PS, n);
            lina::dev::d2d(R, S, n);
            lina::dev::axpy(R, -omega, APS, n);
            double beta = lina::dev::dot(R, R0, n) * alpha / (h * omega);
            lina::dev::axpy(P, -omega, APP, n);
            lina::dev::scal(P, beta, n);
            lina::dev::axpy(P, 1., R, n);
            r = sqrt(lina::dev::dot(R, R, n));
            iter++;
            if (bi_info == BI_YES) printf("\tBiCGStab residuum: %e\n", r / r0);
        } while (r / r0 > bi_eps && iter <= bi_max_iter);
    }
    if (iter == bi_max_iter) printf("BiCGStab: no convergence in %d iterations\n\n", iter);
    AMG_add_stat(&bi_stat, iter, fabs(r / r0));
    if (!lina::dev::d2h(X, x, n)) return -1;
    return iter;
}

}  // extern "C"

// ============================================================ device BiCGStab and ILU(0) (C-ABI)
extern "C" {

int lina_gpu_bicgstab(lina_gpu_matrix* Am, lina_gpu_ilu* ilu, int ilu_precision, const double* b_in, double* x_out,
                      double tol, int max_iter, int flags, lina_gpu_solve_info* info) {
    if (!Am || !b_in || !x_out || max_iter < 0) return LINA_GPU_EINVAL;
    lina_gpu_solve_info local{};
    lina_gpu_solve_info* inf = info ? info : &local;
    memset(inf, 0, sizeof *inf);
    const bool dev = (flags & LINA_PCG_DEVICE_PTRS) != 0;
    const int n = lina_gpu_matrix_rows(Am);
    DevVecs d(10, n);
    if (!d.ok()) return LINA_GPU_ECUDA;
    double *x = d.v[0], *bb = d.v[1], *S = d.v[2], *PS = d.v[3], *PP = d.v[4], *APP = d.v[5], *APS = d.v[6],
           *R = d.v[7], *R0 = d.v[8], *P = d.v[9];
    bool ok = dev ? lina::dev::d2d(bb, b_in, n) : lina::dev::h2d(bb, b_in, n);
    if (flags & LINA_PCG_USE_X0)
        ok = ok && (dev ? lina::dev::d2d(x, x_out, n) : lina::dev::h2d(x, x_out, n));
    else
        ok = ok && lina::dev::zero(x, n);
    auto matvec = [&](const double* in, double* out) {
        lina::dev::sync();
        return lina_gpu_matrix_spmv(Am, LINA_PREC_FP64, in, out) == 0;
    };
    auto precon = [&](const double* in, double* out) {
        lina::dev::sync();
        if (!ilu) return lina::dev::d2d(out, in, n);
        return lina_gpu_ilu_apply(ilu, ilu_precision, in, out) == 0;
    };
    ok = ok && matvec(x, R);
    ok = ok && lina::dev::axpy(R, -1., bb, n) && lina::dev::scal(R, -1., n) && lina::dev::d2d(R0, R, n) &&
         lina::dev::d2d(P, R, n);
    if (!ok) return LINA_GPU_ECUDA;
    double r0 = sqrt(lina::dev::dot(R, R, n)), r = r0;
    int iter = 0;
    if (r0 != 0) {
        do {
            if (!precon(P, PP) || !matvec(PP, APP)) return LINA_GPU_ECUDA;
            double h = lina::dev::dot(R, R0, n);
            double t = lina::dev::dot(APP, R0, n);
            if (t == 0) break;
            double alpha = h / t;
            lina::dev::d2d(S, R, n);
            lina::dev::axpy(S, -alpha, APP, n);
            if (!precon(S, PS) || !matvec(PS, APS)) return LINA_GPU_ECUDA;
            double s = lina::dev::dot(APS, APS, n);
            if (s == 0) break;
            double omega = lina::dev::dot(APS, S, n) / s;
            lina::dev::axpy(x, alpha, PP, n);
            lina::dev::axpy(x, omega, PS, n);
            lina::dev::d2d(R, S, n);
            lina::dev::axpy(R, -omega, APS, n);
            double beta = lina::dev::dot(R, R0, n) * alpha / (h * omega);
            lina::dev::axpy(P, -omega, APP, n);
            lina::dev::scal(P, beta, n);
            lina::dev::axpy(P, 1., R, n);
            r = sqrt(lina::dev::dot(R, R, n));
            iter++;
            if (!std::isfinite(r)) break;
        } while (r / r0 > tol && iter <= max_iter);
    }
    inf->iterations = iter;
    inf->rel_residual = (r0 != 0) ? r / r0 : 0.0;
    if (!std::isfinite(inf->rel_residual))
        inf->status = LINA_GPU_EBREAKDOWN;
    else if (inf->rel_residual > tol)
        inf->status = LINA_GPU_ENOCONV;
    // true residual
    if (!matvec(x, APP)) return LINA_GPU_ECUDA;
    lina::dev::d2d(S, bb, n);
    lina::dev::axpy(S, -1., APP, n);
    double bn = sqrt(lina::dev::dot(bb, bb, n));
    inf->true_rel_residual = bn > 0 ? sqrt(lina::dev::dot(S, S, n)) / bn : 0.0;
    ok = dev ? lina::dev::d2d(x_out, x, n) : lina::dev::d2h(x_out, x, n);
    lina::dev::sync();
    return ok ? inf->status : LINA_GPU_ECUDA;
}

}  // extern "C"

// ============================================================ local solvers for the caller's solver slots
// The reference's callers hand a whole linear solve to a function int f(sparse_matrix* A, double* X,
// double* b): reflective_newton's RN_set_local_solver slot (reflective_newton.c:308), active_set_solver's
// Solver (linear_algebra.c:4995), and Crack/crack.c's UMFPACK wrapper multifrontal_solver (:5424, used by
// the elastic step :9340 and, through multifrontal_solver_AS, the chemical step's active-set solver
// :9250).  These two functions fill such slots on the GPU.  They return POSITIVE_DEFINITE (1) when the
// solve reached its tolerance and INDEFINITE (0) otherwise, the convention of the RN slot.
namespace {

struct SpdCache {
    lina_gpu_amg* h = nullptr;
    int n = 0;
    uint64_t pattern = 0;
    int dof = 0;
} g_spd;

uint64_t pattern_fingerprint(const sparse_matrix* A) {
    uint64_t h = 1469598103934665603ull ^ (uint64_t)A->size;
    for (int i = 0; i < A->size; i++) {
        h = (h ^ (uint64_t)A->Len[i]) * 1099511628211ull;
        for (int k = 0; k < A->Len[i]; k++) h = (h ^ (uint64_t)(uint32_t)A->Indices[i][k]) * 1099511628211ull;
    }
    return h;
}

// levels of the hierarchy for an n-row system: coarsen until a few thousand rows remain
int spd_depth(int n) {
    int d = 1;
    for (double m = n; m > 4000.0 && d < 12; m /= 2.6) d++;
    return d < 2 ? 2 : d;
}

}  // namespace

extern "C" {

/* A X = b for symmetric positive definite A (an elasticity or reaction-diffusion step, the scaled Newton
   matrix of reflective_newton) by AMG-preconditioned CG on the GPU: standard coarsening with the unknowns
   per node of AMG_set_deg_of_freedom, mixed precision, X as initial guess, to ||b - A X|| <= 1e-10 ||b||.
   The hierarchy is kept between calls and rebuilt only when A's pattern changes; new values on the same
   pattern recompute its coarse levels (AMG_recompute_coarse_matrices). */
int LinA_gpu_spd_solver(sparse_matrix* A, double* X, double* b) {
    if (!A || !X || !b || A->size <= 0) return INDEFINITE;
    CsrCopy c = to_csr(A);
    const uint64_t pat = pattern_fingerprint(A);
    int rc = 0;
    if (g_spd.h && g_spd.n == c.n && g_spd.pattern == pat && g_spd.dof == amg_dof) {
        rc = lina_gpu_amg_recompute(g_spd.h, c.n, c.ptr.data(), c.col.data(), c.val.data());
    } else {
        if (g_spd.h) lina_gpu_amg_destroy(g_spd.h);
        g_spd = SpdCache();
        lina_gpu_amg_options o;
        lina_gpu_default_options(&o);
        o.dof = amg_dof > 0 && c.n % amg_dof == 0 ? amg_dof : 1;
        o.depth = spd_depth(c.n);
        o.coarsening = LINA_STANDARD;
        o.smoother = LINA_SMOOTHER_JACOBI;
        o.omega = 0.6;
        o.precision = LINA_PREC_MIXED;
        rc = lina_gpu_amg_create(c.n, c.ptr.data(), c.col.data(), c.val.data(), &o, &g_spd.h);
        if (rc == 0) {
            g_spd.n = c.n;
            g_spd.pattern = pat;
            g_spd.dof = amg_dof;
        } else {
            g_spd.h = nullptr;
        }
    }
    if (rc != 0) {
        fprintf(stderr, "LinA-GB300: LinA_gpu_spd_solver: set-up failed: %s\n", lina_gpu_last_error());
        return INDEFINITE;
    }
    lina_gpu_solve_info info;
    rc = lina_gpu_pcg(g_spd.h, b, X, 1e-10, 5000, LINA_STOP_RELATIVE, LINA_PCG_USE_X0, &info);
    return rc == 0 ? POSITIVE_DEFINITE : INDEFINITE;
}

/* A X = b for a general square A (nonsymmetric, or the indefinite KKT systems active_set_solver builds)
   by restarted GMRES(30) on the GPU with ILU(0) of A as right preconditioner (none where the incomplete
   factorisation meets a zero pivot), X as initial guess, to a relative residual of 1e-10. */
int LinA_gpu_general_solver(sparse_matrix* A, double* X, double* b) {
    if (!A || !X || !b || A->size <= 0) return INDEFINITE;
    lina_gpu_matrix* m = device_matrix(A);
    if (!m) return INDEFINITE;
    CsrCopy c = to_csr(A);
    lina_gpu_ilu* ilu = nullptr;
    if (lina_gpu_ilu_create_from_matrix(c.n, c.ptr.data(), c.col.data(), c.val.data(), &ilu) != 0) ilu = nullptr;
    lina_gpu_solve_info info;
    // GMRES works on the preconditioned unknown y (x = B_r y); start from y = 0 and return x
    std::vector<double> y(c.n, 0.0);
    int rc = lina_gpu_gmres(m, ilu, nullptr, LINA_PREC_FP64, b, y.data(), 1e-10, 30, 20000, 1,
                            LINA_GMRES_APPLY_PRECON, &info);
    if (ilu) lina_gpu_ilu_destroy(ilu);
    if (rc != 0 && rc != LINA_GPU_ENOCONV) return INDEFINITE;
    for (int i = 0; i < c.n; i++) X[i] = y[i];
    return rc == 0 ? POSITIVE_DEFINITE : INDEFINITE;
}

}  // extern "C"
