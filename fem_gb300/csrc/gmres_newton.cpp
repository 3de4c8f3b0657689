// gmres_newton.cpp - the gmres entry point, the finite-difference Newton
// solver (LinA/GMRES_Newton.c:34-295) and the active-set solver
// (LinA/linear_algebra.c:4933-5042) with the row-list helpers they use.
//
// gmres runs the device GMRES of gpu_gmres.cu; the caller's product and
// preconditioners are applied to device vectors, on the GPU when they are the
// library's own (including the Newton solver's Jacobian product and ILU(0)
// preconditioner), on host copies otherwise.  Newton_solver and
// active_set_solver are host loops around those solves, as in the reference.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "BiCGStab.h"
#include "GMRES_Newton.h"
#include "PCGS.h"
#include "gmres_gpu.h"
#include "gpu_ops.h"
#include "itlin.h"
#include "lina_gpu.h"
#include "lina_internal.h"
#include "linear_algebra.h"

// ============================================================ row-list helpers
extern "C" {

void copy_vector_content(double* x, double* y, int x_pos, int y_pos, int size) {
    for (int i = x_pos; i < x_pos + size; i++) y[y_pos - x_pos + i] = x[i];
}

int* clone_list(int* x, int n) {
    int* r = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
    for (int i = 0; i < n; i++) r[i] = x[i];
    return r;
}

int* zero_int_list(int n) {
    int* r = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
    for (int i = 0; i < n; i++) r[i] = 0;
    return r;
}

double* generate_vector(int size, double val) {
    double* r = (double*)malloc((size > 0 ? size : 1) * sizeof(double));
    for (int i = 0; i < size; i++) r[i] = val;
    return r;
}

void vector_pseudo_mult(double* x, double* y, int n) {
    for (int i = 0; i < n; i++) x[i] *= y[i];
}

// linear_algebra.c:4109: grow A to new_size rows; row/column block l of width mesh_size moves to
// block l + equ_index / l + var_index; the new rows hold the (i, 0.0) placeholder
void enlarge_matrix(sparse_matrix* A, int mesh_size, int new_size, int equ_index, int var_index) {
    const int old = A->size;
    A->Len = (int*)realloc(A->Len, new_size * sizeof(int));
    A->Indices = (int**)realloc(A->Indices, new_size * sizeof(int*));
    A->Values = (double**)realloc(A->Values, new_size * sizeof(double*));
    A->size = new_size;
    for (int i = 0; i < old; i++)
        for (int j = 0; j < A->Len[i]; j++) {
            const int k = A->Indices[i][j] % mesh_size, l = A->Indices[i][j] / mesh_size;
            A->Indices[i][j] = (l + var_index) * mesh_size + k;
        }
    for (int i = old - 1; i >= 0; i--) {
        const int t = (i / mesh_size + equ_index) * mesh_size + i % mesh_size;
        A->Indices[t] = A->Indices[i];
        A->Values[t] = A->Values[i];
        A->Len[t] = A->Len[i];
    }
    for (int i = 0; i < new_size; i++)
        if (i < equ_index * mesh_size || i >= equ_index * mesh_size + old) {
            A->Len[i] = 1;
            A->Indices[i] = (int*)malloc(sizeof(int));
            A->Values[i] = (double*)malloc(sizeof(double));
            A->Indices[i][0] = i;
            A->Values[i][0] = 0;
        }
}

void simple_enlarge_matrix(sparse_matrix* A, int add_size) {
    const int n = A->size, m = n + add_size;
    A->size = m;
    A->Len = (int*)realloc(A->Len, m * sizeof(int));
    A->Indices = (int**)realloc(A->Indices, m * sizeof(int*));
    A->Values = (double**)realloc(A->Values, m * sizeof(double*));
    for (int i = n; i < m; i++) {
        A->Len[i] = 1;
        A->Indices[i] = (int*)malloc(sizeof(int));
        A->Values[i] = (double*)malloc(sizeof(double));
        A->Indices[i][0] = i;
        A->Values[i][0] = 0;
    }
}

// dense LU without pivoting (Doolittle: L unit lower, U upper); rows of L and U are allocated here
void LU_factorzation(double** A, double** L, double** U, int size) {
    for (int i = 0; i < size; i++) {
        L[i] = (double*)calloc(size, sizeof(double));
        U[i] = (double*)calloc(size, sizeof(double));
    }
    for (int k = 0; k < size; k++) {
        for (int j = k; j < size; j++) {
            double s = A[k][j];
            for (int p = 0; p < k; p++) s -= L[k][p] * U[p][j];
            U[k][j] = s;
        }
        L[k][k] = 1.0;
        for (int i = k + 1; i < size; i++) {
            double s = A[i][k];
            for (int p = 0; p < k; p++) s -= L[i][p] * U[p][k];
            L[i][k] = s / U[k][k];
        }
    }
}

// linear_algebra.c:3040: dense LU of the rows with more than one nonzero (and their columns),
// rows with one nonzero become L_ii = 1, U_ii = a_ii
void sparse_LU_factorization(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U) {
    const int n = A->size;
    std::vector<int> map(n, -1), inv;
    for (int i = 0; i < n; i++) {
        int nz = 0;
        for (int j = 0; j < A->Len[i]; j++) nz += A->Values[i][j] != 0 ? 1 : 0;
        if (nz > 1) {
            map[i] = (int)inv.size();
            inv.push_back(i);
        }
    }
    const int m = (int)inv.size();
    std::vector<double*> S(m), SL(m), SU(m);
    for (int I = 0; I < m; I++) {
        S[I] = (double*)calloc(m > 0 ? m : 1, sizeof(double));
        const int i = inv[I];
        for (int j = 0; j < A->Len[i]; j++) {
            const int J = map[A->Indices[i][j]];
            if (J >= 0) S[I][J] = A->Values[i][j];
        }
    }
    LU_factorzation(S.data(), SL.data(), SU.data(), m);
    for (int I = 0; I < m; I++)
        for (int J = 0; J < m; J++) {
            if (SL[I][J] != 0) insert_sparse(L, SL[I][J], inv[I], inv[J]);
            if (SU[I][J] != 0) insert_sparse(U, SU[I][J], inv[I], inv[J]);
        }
    for (int i = 0; i < n; i++)
        if (map[i] < 0) {
            insert_sparse(L, 1., i, i);
            insert_sparse(U, get_diag(A, i), i, i);
        }
    for (int I = 0; I < m; I++) {
        free(S[I]);
        free(SL[I]);
        free(SU[I]);
    }
}

// linear_algebra.c:3122: dense LU of the whole matrix, nonzeros copied into L and U
void complete_LU_factorization(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U) {
    const int n = A->size;
    std::vector<double*> M(n), LA(n), UA(n);
    for (int i = 0; i < n; i++) {
        M[i] = (double*)calloc(n, sizeof(double));
        for (int j = 0; j < A->Len[i]; j++) M[i][A->Indices[i][j]] = A->Values[i][j];
    }
    LU_factorzation(M.data(), LA.data(), UA.data(), n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            if (LA[i][j] != 0) insert_sparse(L, LA[i][j], i, j);
            if (UA[i][j] != 0) insert_sparse(U, UA[i][j], i, j);
        }
    for (int i = 0; i < n; i++) {
        free(M[i]);
        free(LA[i]);
        free(UA[i]);
    }
}

}  // extern "C"

// ============================================================ gmres
namespace {

// Newton solver state (GMRES_Newton.c:5-33)
const double kNewtonStep = 1e-6;
sparse_matrix* newton_matrix = nullptr;
sparse_matrix* newton_L = nullptr;
sparse_matrix* newton_U = nullptr;
sparse_matrix* newton_pattern = nullptr;
double** newton_roots = nullptr;
double* newton_B = nullptr;
int newton_B_size = 0;
int newton_root_number = 0;
double *search_min = nullptr, *search_max = nullptr, *range_min = nullptr, *range_max = nullptr;
int newton_guesses = 10000;
ITLIN_OPT* newton_opt = nullptr;
ITLIN_INFO* newton_info = nullptr;
double (*newton_F)(double* X, int i, int size) = nullptr;

// the Jacobian product and its ILU(0) preconditioner (GMRES_Newton.c:94-111); inside gmres they
// run on the GPU
void Newton_matvec(int n, double* y, double* z) {
    for (int i = 0; i < n; i++) {
        double s = 0;
        for (int j = 0; j < newton_matrix->Len[i]; j++) s += newton_matrix->Values[i][j] * y[newton_matrix->Indices[i][j]];
        z[i] = s;
    }
}

void Newton_preconlr(int n, double* z, double* w) {
    copy_vector_content(z, w, 0, 0, n);
    L_triang_invert(newton_L, w);
    U_triang_invert(newton_U, w);
}

struct HostStage {
    std::vector<double> a, b;
    void ensure(int n) {
        if ((int)a.size() < n) a.resize(n), b.resize(n);
    }
} g_stage;

// a PRECON of the gmres interface as an operator on device vectors (empty: identity)
lina::gm::Op precon_op(PRECON* f, int n) {
    if (!f) return lina::gm::Op();
    if (f == Newton_preconlr)
        return [n](const double* x, double* y) {
            lina_gpu_ilu* ilu = lina::api::device_ilu(newton_L, newton_U);
            if (!ilu) return false;
            lina::dev::sync();
            return lina_gpu_ilu_apply(ilu, LINA_PREC_FP64, x, y) == 0;
        };
    auto pf = reinterpret_cast<lina::api::PreconFn>(f);
    if (pf == PCG_preconlr || pf == PCG_AMG_precon || pf == BI_AMG_precon)
        return [pf, n](const double* x, double* y) { return lina::api::device_precon(pf, n, x, y) >= 0; };
    return [f, n](const double* x, double* y) {
        g_stage.ensure(n);
        if (!lina::dev::d2h(g_stage.a.data(), x, n) || !lina::dev::d2h(g_stage.b.data(), y, n)) return false;
        f(n, g_stage.a.data(), g_stage.b.data());
        return lina::dev::h2d(y, g_stage.b.data(), n);
    };
}

lina::gm::Op matvec_op(MATVEC* f, int n) {
    if (f == Newton_matvec)
        return [n](const double* x, double* y) {
            lina_gpu_matrix* m = lina::api::device_matrix(newton_matrix);
            if (!m) return false;
            lina::dev::sync();
            return lina_gpu_matrix_spmv(m, LINA_PREC_FP64, x, y) == 0;
        };
    return [f, n](const double* x, double* y) { return lina::api::device_matmult(f, n, x, y); };
}

}  // namespace

extern "C" void gmres(int n, double* y, MATVEC* matvec, PRECON* preconr, PRECON* preconl, double* b,
                      struct ITLIN_OPT* opt, struct ITLIN_INFO* info) {
    FILE* err = (opt && opt->errorfile) ? opt->errorfile : stdout;
    const bool verbose = opt && opt->errorlevel > 0;
    info->iter = 0;
    info->nomatvec = info->noprecl = info->noprecr = 0;
    info->precision = 0;
    // parameter checks and defaults (the NewtonLib rules)
    if (!matvec) {
        if (verbose) fprintf(err, "\n Error - Routine matvec must be supplied\n");
        info->rcode = -99;
        return;
    }
    if (n <= 0) {
        if (verbose) fprintf(err, "\n Error - Number of Equations/unknowns must be >0\n");
        info->rcode = 20;
        return;
    }
    if (opt->tol <= 0) {
        if (verbose) fprintf(err, "\n Error - opt->tol must be positive\n");
        info->rcode = 21;
        return;
    }
    if (opt->tol > 1e-1) opt->tol = 1e-1;
    if (opt->tol < 1e-15) opt->tol = 1e-15;
    if (opt->i_max <= 0 || opt->i_max > n) opt->i_max = n < 10 ? n : 10;
    const int max_iter = opt->maxiter <= 0 ? 100 : opt->maxiter;
    double* dy = lina::dev::alloc(n);
    double* db = lina::dev::alloc(n);
    lina::gm::Result r;
    bool ok = dy && db && lina::dev::h2d(dy, y, n) && lina::dev::h2d(db, b, n);
    ok = ok && lina::gm::solve(n, dy, db, matvec_op(matvec, n), precon_op(preconr, n), precon_op(preconl, n), opt->tol,
                               opt->i_max, max_iter, opt->termcheck == CheckEachIter, r);
    ok = ok && lina::dev::d2h(y, dy, n);
    lina::dev::release(dy);
    lina::dev::release(db);
    if (!ok) {
        fprintf(stderr, "LinA-GB300: gmres: device failure: %s\n", lina_gpu_last_error());
        info->rcode = -999;
        return;
    }
    info->rcode = r.rcode;
    info->precision = r.precision;
    info->iter = r.iter;
    info->nomatvec = r.nomatvec;
    info->noprecl = r.noprecl;
    info->noprecr = r.noprecr;
    if (verbose && r.rcode == 2) fprintf(err, "\n Error - Maximum allowed number of iterations exceeded size: %d\n", n);
    if (verbose && r.rcode == 1) fprintf(err, "\n Error, code=%i\n", r.rcode);
}

// ============================================================ Newton solver
namespace {

double mod_F(double* X, int i, int size) {
    double pro = 1.;
    for (int r = 0; r < newton_root_number; r++) {
        double s = 0;
        for (int j = 0; j < newton_pattern->Len[i]; j++) {
            const int k = newton_pattern->Indices[i][j];
            s += (X[k] - newton_roots[r][k]) * (X[k] - newton_roots[r][k]);
        }
        pro *= s;
    }
    return newton_F(X, i, size) / sqrt(pro);
}

double b_at(int i) { return (newton_B && i < newton_B_size) ? newton_B[i] : 0.0; }

void set_residuum(double* X, double* Y, int size) {
    for (int i = 0; i < size; i++) Y[i] = b_at(i) - mod_F(X, i, size);
}

sparse_matrix* sparse_jacobian(sparse_matrix* P, double* X) {
    const int n = P->size;
    sparse_matrix* J = sparse_zero(n);
    for (int i = 0; i < n; i++) {
        const double f0 = mod_F(X, i, n);
        for (int j = 0; j < P->Len[i]; j++)
            if (P->Values[i][j] != 0) {
                const int k = P->Indices[i][j];
                X[k] += kNewtonStep;
                insert_sparse(J, (mod_F(X, i, n) - f0) / kNewtonStep, i, k);
                X[k] -= kNewtonStep;
            }
    }
    return J;
}

bool in_range(double* X) {
    if (!range_min || !range_max) return true;
    for (int i = 0; i < newton_pattern->size; i++)
        if (X[i] < range_min[i] || X[i] > range_max[i]) return false;
    return true;
}

}  // namespace

extern "C" {

void Newton_GMRES_options(int bases_imax, int maxiter, double tol) {
    newton_opt = (ITLIN_OPT*)calloc(1, sizeof(ITLIN_OPT));
    newton_opt->tol = tol;
    newton_opt->i_max = bases_imax;
    newton_opt->maxiter = maxiter;
    newton_opt->termcheck = CheckOnRestart;
    newton_opt->errorlevel = Verbose;
    newton_opt->monitorlevel = None;
    newton_opt->datalevel = None;
    newton_opt->errorfile = stdout;
    newton_opt->monitorfile = stdout;
    newton_info = (ITLIN_INFO*)calloc(1, sizeof(ITLIN_INFO));
}

void Newton_first_guess_options(int guess_num, int size, double* Min, double* Max) {
    newton_guesses = guess_num;
    if (!search_min) search_min = zero_vector(size);
    if (!search_max) search_max = zero_vector(size);
    for (int i = 0; i < size; i++) search_min[i] = Min[i], search_max[i] = Max[i];
}

void Newton_set_range(int size, double* Min, double* Max) {
    if (!range_min) range_min = zero_vector(size);
    if (!range_max) range_max = zero_vector(size);
    for (int i = 0; i < size; i++) range_min[i] = Min[i], range_max[i] = Max[i];
}

void Newton_set_function(double (*F)(double* X, int i, int size)) { newton_F = F; }

void Newton_set_inhomo(double* B, int n) {
    if (!newton_B) {
        newton_B = zero_vector(n);
        newton_B_size = n;
    }
    if (B)
        for (int i = 0; i < n; i++) newton_B[i] = B[i];
}

sparse_matrix* Newton_get_full_pattern(int size) {
    sparse_matrix* R = sparse_zero(size);
    for (int i = 0; i < size; i++)
        for (int j = 0; j < size; j++) insert_sparse(R, 1., i, j);
    return R;
}

double** Newton_get_all_roots(void) {
    const int n = newton_pattern ? newton_pattern->size : 0;
    double** R = (double**)malloc((newton_root_number > 0 ? newton_root_number : 1) * sizeof(double*));
    for (int i = 0; i < newton_root_number; i++) {
        R[i] = clone_vector(newton_roots[i], n);
        free(newton_roots[i]);
    }
    free(newton_roots);
    newton_roots = nullptr;
    return R;
}

// the best of newton_guesses uniform random points in the search box (rand(), unseeded as in the
// reference)
void Newton_first_guess(double* Res, int n) {
    std::vector<double> guess(n), value(n);
    double r_min = DBL_MAX;
    for (int g = 0; g < newton_guesses; g++) {
        for (int j = 0; j < n; j++)
            guess[j] = (double)search_min[j] + rand() * (search_max[j] - search_min[j]) / RAND_MAX;
        for (int j = 0; j < n; j++) value[j] = mod_F(guess.data(), j, n) - b_at(j);
        const double r = euklid_norm(value.data(), n);
        if (r < r_min) {
            r_min = r;
            copy_vector_content(guess.data(), Res, 0, 0, n);
        }
    }
}

int Newton_solver(sparse_matrix* Pattern, double* X, double maxiter, double eps, int mode, double r0) {
    const int n = Pattern->size;
    std::vector<double> R(n, 0.0);
    newton_pattern = Pattern;
    if (r0 < 0) {
        set_residuum(X, R.data(), n);
        r0 = euklid_norm(R.data(), n);
    }
    if (mode == LARGE_SYSTEM && !newton_opt) Newton_GMRES_options(30, 1000, 1e-8);
    double r = r0;
    int i = 0;
    if (r0 != 0) do {
            newton_matrix = sparse_jacobian(newton_pattern, X);
            newton_L = sparse_zero(n);
            newton_U = sparse_zero(n);
            std::vector<double> H(n, 0.0);
            bool gave_up = false;
            if (mode == LARGE_SYSTEM) {
                incomplete_LU_factorization(newton_matrix, newton_L, newton_U);
                gmres(n, H.data(), Newton_matvec, Newton_preconlr, nullptr, R.data(), newton_opt, newton_info);
                if (newton_info->iter >= newton_opt->maxiter) gave_up = true;
            } else {
                sparse_LU_factorization(newton_matrix, newton_L, newton_U);
                H = R;
            }
            if (!gave_up) {
                L_triang_invert(newton_L, H.data());
                U_triang_invert(newton_U, H.data());
                vector_add(X, H.data(), 1., n);
                set_residuum(X, R.data(), n);
                r = euklid_norm(R.data(), n);
            }
            lina::api::forget_device_matrix(newton_matrix);
            free_sparse(newton_matrix);
            free_sparse(newton_L);
            free_sparse(newton_U);
            newton_matrix = newton_L = newton_U = nullptr;
            if (gave_up) {
                i = (int)maxiter;
                break;
            }
            if (std::isnan(r)) {
                printf("Newton Warning: singular Jacobian\n");
                printf("Newton residuum reduction: %e\n", r / r0);
                return -1;
            }
            if (!in_range(X)) {
                Newton_first_guess(X, n);
                set_residuum(X, R.data(), n);
                r = euklid_norm(R.data(), n);
            }
            i++;
        } while (i < maxiter && r / r0 > eps);
    if (i == (int)maxiter) {
        printf("GMRES Newton: no convergence with given tolerance\n -> abort\n");
        return -1;
    }
    if (i != 0)
        printf("GMRES Newton: residuum reduction: %f ; %d iterations\n", r / r0, i);
    else
        printf("GMRES Newton: initial residuum equals zero -> continue ...\n");
    return i;
}

int Newton_solver_mult_Root(sparse_matrix* Pattern, double maxiter, double eps, int mode) {
    const int n = Pattern->size;
    std::vector<double> guess(n, 0.0), R(n, 0.0);
    newton_pattern = Pattern;
    newton_root_number = 0;
    set_residuum(guess.data(), R.data(), n);
    int iter;
    do {
        Newton_first_guess(guess.data(), n);
        iter = Newton_solver(Pattern, guess.data(), maxiter, eps, mode, euklid_norm(R.data(), n));
        if (iter >= 0 && iter < maxiter) {
            newton_root_number++;
            newton_roots = (double**)realloc(newton_roots, newton_root_number * sizeof(double*));
            newton_roots[newton_root_number - 1] = clone_vector(guess.data(), n);
        }
    } while (iter >= 0 && iter < maxiter);
    return newton_root_number;
}

// ============================================================ active-set solver
// KKT system [A C^T; C 0] with the active constraints (linear_algebra.c:4868, the default form;
// :4886 for ASS_FLUX, which couples the constraint into the second field)
static sparse_matrix* add_constraints(sparse_matrix* A, sparse_matrix* C, int* active, int na, int mode) {
    const int N = A->size, m = C->size;
    sparse_matrix* R = clone(A);
    if (mode == ASS_FLUX) {
        simple_enlarge_matrix(R, na);
        for (int k = 0; k < na; k++) {
            const int i = active[k];
            for (int j = 0; j < C->Len[i]; j++) {
                insert_sparse(R, C->Values[i][j], m + C->Indices[i][j], N + k);
                insert_sparse(R, C->Values[i][j], N + k, C->Indices[i][j]);
            }
        }
        return R;
    }
    sparse_matrix* CT = get_transpose(C, m);
    enlarge_matrix(R, N, N + na, 0, 0);
    for (int k = 0; k < na; k++) {
        const int i = active[k];
        for (int j = 0; j < CT->Len[i]; j++) {
            insert_sparse(R, CT->Values[i][j], CT->Indices[i][j], N + k);
            insert_sparse(R, CT->Values[i][j], N + k, CT->Indices[i][j]);
        }
    }
    free_sparse(CT);
    return R;
}

void free_ass_info(ass_info** info) {
    if (*info) {
        free((*info)->Active);
        free((*info)->Signs);
        free((*info)->Constraint);
        free((*info)->Iter_history);
        free(*info);
    }
}

int active_set_solver(sparse_matrix* A, double* Sol, double* b, sparse_matrix* B, double* L, double* U,
                      int (*Solver)(sparse_matrix* A, double* X, double* b), int max_iter, double definiteness, int mode,
                      ass_info** solver_info) {
    const double tol = 1e-10;
    if (!*solver_info) {
        *solver_info = (ass_info*)calloc(1, sizeof(ass_info));
    }
    ass_info* S = *solver_info;
    const int n = A->size, m = B->size;
    if (!S->Active) S->Active = zero_int_list(m);
    if (!S->Signs) S->Signs = zero_vector(m);
    if (!S->Constraint) S->Constraint = zero_vector(m);
    std::vector<double> Z(b, b + n);
    std::vector<double> X(n + m, 0.0);
    copy_vector_content(Sol, X.data(), 0, 0, n);
    int iter = 0, fulfilled;
    do {
        std::vector<int> act;
        std::vector<double> sg;
        Z.resize(n + S->active_size);
        for (int i = 0; i < m; i++)
            if (S->Active[i]) {
                if ((int)act.size() < S->active_size) Z[n + act.size()] = S->Constraint[i];
                act.push_back(i);
                sg.push_back(S->Signs[i]);
            }
        if ((int)act.size() != S->active_size) printf("\nsomenthing's wrong in active_set_solver\n");
        sparse_matrix* M = add_constraints(A, B, act.data(), S->active_size, mode);
        Solver(M, X.data(), Z.data());
        free_sparse(M);
        fulfilled = 1;
        // multipliers of the wrong sign release their constraints; the loop bound is the live
        // count, so each release shortens the scan, as in the reference
        double* Y = sparse_mult(B, X.data());
        for (int k = 0; k < S->active_size; k++)
            if (sg[k] * X[n + k] * definiteness > 0) {
                S->Active[act[k]] = 0;
                S->active_size--;
                fulfilled = 0;
            }
        // violated bounds become active
        for (int i = 0; i < m; i++)
            if (Y[i] < L[i] - tol || Y[i] > U[i] + tol) {
                if (!S->Active[i]) S->active_size++;
                S->Active[i] = 1;
                if (Y[i] < L[i] - tol) {
                    S->Signs[i] = 1.;
                    S->Constraint[i] = L[i];
                }
                if (Y[i] > U[i] + tol) {
                    S->Signs[i] = -1.;
                    S->Constraint[i] = U[i];
                }
                fulfilled = 0;
            }
        free(Y);
        iter++;
    } while (!fulfilled && iter < max_iter);
    copy_vector_content(X.data(), Sol, 0, 0, n);
    if (iter >= max_iter) printf("Warning: no convergence in %d iterations\n", iter);
    S->Iter_history = (int*)realloc(S->Iter_history, (S->calls + 1) * sizeof(int));
    S->Iter_history[S->calls] = iter;
    S->calls++;
    return iter;
}

}  // extern "C"
