// rn.cpp - reflective Newton for bound-constrained minimisation
// (LinA/reflective_newton.c) with its vectors on the GPU.
//
// The iteration restates reflective_newton / RN_iterate step by step: the
// scaling D and indicator J of the active bounds, the scaled Newton matrix
// M = D H D + diag(|g| J), the local Newton solve, the two-dimensional
// trust-region subspace minimisation, the reflected step with its bisection
// line search, the boundary nudge and the trust-radius update.  Vectors live
// on the GPU (elementwise kernels in rn_kernels.cu, BLAS-1 in gpu_ops.cu);
// the caller's functional, gradient and Hessian callbacks receive host copies
// of the iterate, as they are host functions.  The default quadratic
// functional q(x) = x.H.x/2 + x.b and its gradient run on the GPU.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gpu_ops.h"
#include "lina_gpu.h"
#include "lina_internal.h"
#include "reflective_newton.h"
#include "rn_gpu.h"

namespace {

// settings (reflective_newton.c:5-16)
int rn_max_iter = 50;
double rn_eps = 1e-8;
double rn_sigma_l = 0.1;
double rn_sigma_u = 0.9;
double rn_rho = 0.1;
double rn_Delta = 250.;
double rn_Xi = 1.;
double rn_trust_lower = 0.6;
double rn_trust_upper = 1.1;
double rn_trust_radius_min = 1e-3;
double rn_trust_radius_max = 1000.;

int rn_solver_type = RN_BICGSTAB;
RN_statistics stats;
int rn_pcg_iter = 100;
const int eig_iter = 10000;
const double eig_eps = 1e-6;

int rn_dim = 0;
int* rn_bound = nullptr;
int rn_bound_num = 0;
int rn_status = POSITIVE_DEFINITE;
double* rn_upper = nullptr;
double* rn_lower = nullptr;
double rn_ax = 0, rn_ay = 0, rn_axy = 0, rn_bx = 0, rn_by = 0;

int (*rn_local_solver)(sparse_matrix*, double*, double*) = nullptr;
double (*rn_functional)(double*, int) = nullptr;
double* (*rn_gradient)(double*) = nullptr;
sparse_matrix* (*rn_compute_hesse)(double*) = nullptr;
sparse_matrix* rn_hesse = nullptr;
sparse_matrix* rn_M = nullptr;
double* rn_b = nullptr;
double* kernel_dir = nullptr;
amg_system_info* rn_amg = nullptr;
int rn_info = RN_YES;

}  // namespace

sparse_matrix* lina::api::rn_default_matrix() { return rn_M; }

extern "C" {

void RN_print_info(int mode) { rn_info = mode; }
void RN_set_debug_mode(int mode) { (void)mode; }
int RN_info_set(void) { return rn_info; }

void RN_set_params(int max_iter, double eps, double sigma_l, double sigma_u, double rho, double Delta, double Xi,
                   double trust_lower, double trust_upper, double trust_radius_min, double trust_radius_max) {
    rn_max_iter = max_iter;
    rn_eps = eps;
    rn_sigma_l = sigma_l;
    rn_sigma_u = sigma_u;
    rn_rho = rho;
    rn_Delta = Delta;
    rn_Xi = Xi;
    rn_trust_lower = trust_lower;
    rn_trust_upper = trust_upper;
    rn_trust_radius_min = trust_radius_min;
    rn_trust_radius_max = trust_radius_max;
}

void set_RN_params(int max_iter, double eps, double sigma_l, double sigma_u) {
    rn_max_iter = max_iter;
    rn_eps = eps;
    rn_sigma_l = sigma_l;
    rn_sigma_u = sigma_u;
}

void RN_set_trust_region(double Delta) { rn_Delta = Delta; }
void RN_set_trust_limits(double mn, double mx) {
    rn_trust_radius_min = mn;
    rn_trust_radius_max = mx;
}

void RN_init_statistics(void) { memset(&stats, 0, sizeof stats); }

void print_RN_statistics(FILE* file) {
    if (stats.total_iter != 0 && stats.number_neg_curv != 0)
        stats.average_eig_iter = stats.average_eig_iter / stats.number_neg_curv;
    if (stats.line_search_count != 0) stats.line_search_iter = stats.line_search_iter / stats.line_search_count;
    fprintf(file, "\nReflective Newton statistics:\n");
    fprintf(file, "average number of Newton iterations: %f\n", stats.calls ? (float)stats.total_iter / stats.calls : 0.f);
    fprintf(file, "average residual: %e\n", stats.calls ? (float)stats.res / stats.calls : 0.f);
    fprintf(file, "number of neg. curvature events: %d\n", stats.number_neg_curv);
    fprintf(file, "line searches: %d\n", stats.line_search_count);
    if (stats.line_search_count != 0)
        fprintf(file, "\taverage line search iterations: %d\n\n", stats.line_search_iter);
}

void RN_set_default_matrix(sparse_matrix* M) { rn_M = M; }

// z = M y with the matrix of RN_set_default_matrix, on the GPU
void RN_default_mat_mult(int n, double* y, double* z) {
    if (!rn_M) {
        printf("error in mat_mult: no system matrix set -> abort\n");
        return;
    }
    lina_gpu_matrix* m = lina::api::device_matrix(rn_M);
    double* dy = lina::dev::alloc(n);
    double* dz = lina::dev::alloc(n);
    if (m && dy && dz && lina::dev::h2d(dy, y, n) && lina_gpu_matrix_spmv(m, LINA_PREC_FP64, dy, dz) == 0)
        lina::dev::d2h(z, dz, n);
    lina::dev::release(dy);
    lina::dev::release(dz);
}

void RN_set_Hesse_function(sparse_matrix* (*Hesse_func)(double* X), int dim_Hesse) {
    rn_compute_hesse = Hesse_func;
    rn_dim = dim_Hesse;
    rn_hesse = nullptr;
}

void RN_set_gradient(double* (*Gradient_func)(double* X)) { rn_gradient = Gradient_func; }
void RN_set_AMG_data(amg_system_info* info) { rn_amg = info; }

void RN_set_local_solver(int (*Solver)(sparse_matrix* A, double* X, double* b)) {
    rn_local_solver = Solver;
    if (Solver) rn_solver_type = RN_UMF;
}

void RN_set_solver(int type) { rn_solver_type = type; }

void RN_set_kernel(double* K, int n) {
    if (n == rn_dim)
        kernel_dir = K;
    else
        printf("kernel vector dimension does not match system dimension -> abort\n");
}

int* get_all_indices(int size) {
    int* r = (int*)malloc((size > 0 ? size : 1) * sizeof(int));
    for (int i = 0; i < size; i++) r[i] = i;
    return r;
}

void set_RN_constraints(int* Index_set, double* Lower, double* Upper, int n) {
    rn_bound = Index_set;
    rn_bound_num = n;
    rn_lower = Lower;
    rn_upper = Upper;
    if (rn_info == YES)
        for (int i = 0; i < n; i++)
            if (Lower[i] == Upper[i]) printf("Reflective Newton: upper==lower at index %d -> use Dirichlet\n", i);
}

void set_RN_functional(double (*F)(double* X, int n)) { rn_functional = F; }

void set_RN_Hesse(sparse_matrix* A) {
    rn_hesse = A;
    if (A) rn_dim = A->size;
}

void set_RN_linear(double* B) { rn_b = B; }

}  // extern "C"

// ============================================================ one-dimensional root finders
// (GMRES_Newton.c:298-440): a secant iteration deflated by the roots already
// found (l'Hospital quotient of F and the root polynomial), and a scan of
// sub-intervals for sign changes that runs it on each bracketing interval.
namespace {

double root_poly(const double* roots, int n, double x) {
    double r = 1.;
    for (int i = 0; i < n; i++) r *= (x - roots[i]);
    return r;
}

double der_F(double (*F)(double), double x, int depth) {
    const double dx = 1e-6;
    if (depth == 0) return F(x);
    return (der_F(F, x + dx, depth - 1) - der_F(F, x - dx, depth - 1)) / (2. * dx);
}

double der_poly(const double* roots, int n, double x, int depth) {
    const double dx = 1e-6;
    if (depth == 0) return root_poly(roots, n, x);
    return (der_poly(roots, n, x + dx, depth - 1) - der_poly(roots, n, x - dx, depth - 1)) / (2. * dx);
}

double F_hospital(double (*F)(double), const double* roots, int n, double x) {
    const double eps = 1e-5;
    int depth = 0;
    double dp, df;
    do {
        dp = der_poly(roots, n, x, depth);
        df = der_F(F, x, depth);
        depth++;
    } while (fabs(dp) < eps && fabs(df) < eps && depth < 64);
    return df / dp;
}

}  // namespace

extern "C" {

int Newton_1D(double (*F)(double x), double** Roots, double min, double max, int max_iter, double eps) {
    int i, root_num = 0;
    double f, x, x0, x1, f0, f1, F0, local_eps;
    do {
        local_eps = eps;
        x0 = min;
        x1 = max;
        f0 = F_hospital(F, *Roots, root_num, x0);
        f1 = F_hospital(F, *Roots, root_num, x1);
        F0 = (f0 != 0) ? f0 : 1.;
        i = 0;
        do {
            x = x1 - f1 * (x1 - x0) / (f1 - f0);
            if (x < min || x > max) {
                double r = (double)rand() / RAND_MAX;
                x = min + (max - min) * r;
            }
            f = F_hospital(F, *Roots, root_num, x);
            x0 = x1;
            x1 = x;
            f0 = f1;
            f1 = f;
            i++;
            if (i == max_iter / 2) local_eps *= 1e2;
        } while (fabs(f / F0) > local_eps && i < max_iter);
        if (i < max_iter) {
            root_num++;
            *Roots = (double*)realloc(*Roots, root_num * sizeof(double));
            (*Roots)[root_num - 1] = x;
        }
    } while (i < max_iter);
    if (root_num == 0) printf("Newton 1D: no roots found in given interval\n");
    return root_num;
}

int Interval_Separation_Newton_1D(double (*F)(double x), double** Roots, double min, double max, int max_iter,
                                  double eps, int int_num) {
    const double d = (max - min) / int_num;
    int root_num = 0;
    *Roots = nullptr;
    for (int i = 0; i < int_num; i++) {
        const double l = i * d, r = l + d;
        const double fl = F(l), fr = F(r);
        if (fl * fr < 0) {
            double* local = nullptr;
            int found = Newton_1D(F, &local, l, r, max_iter, eps);
            if (found > 0) {
                root_num += found;
                *Roots = (double*)realloc(*Roots, root_num * sizeof(double));
                for (int j = 0; j < found; j++) (*Roots)[root_num - j - 1] = local[j];
            }
            free(local);
        } else {
            // the reference records the function value, which is 0, as the root here
            if (fl == 0) {
                root_num++;
                *Roots = (double*)realloc(*Roots, root_num * sizeof(double));
                (*Roots)[root_num - 1] = fl;
            }
            if (fr == 0) {
                root_num++;
                *Roots = (double*)realloc(*Roots, root_num * sizeof(double));
                (*Roots)[root_num - 1] = fr;
            }
        }
    }
    return root_num;
}

}  // extern "C"

// ============================================================ device state of one reflective_newton call
namespace {

using lina::api::CsrCopy;

struct Ctx {
    int n = 0;
    lina::rn::Bounds bounds;
    std::vector<double*> owned;
    double *X = nullptr, *Xold = nullptr, *G = nullptr, *D = nullptr, *J = nullptr, *V1 = nullptr, *V2 = nullptr,
           *B = nullptr, *S = nullptr, *T = nullptr, *T2 = nullptr, *rhs = nullptr, *lin = nullptr;
    std::vector<double> hX, hG, hD, hJ, hA, hB;
    lina_gpu_matrix* H = nullptr;     // device copy of the Hessian (cached by the API layer)
    lina_gpu_matrix* Mdev = nullptr;  // the scaled Newton matrix of this iteration
    CsrCopy Mc;                       // its CSR form
    CsrCopy Hc;                       // the Hessian's CSR form
    sparse_matrix* Mrow = nullptr;    // its row-list form (built only when a solver needs it)
    // the pattern Mdev and ilu were built for: a later step with the same pattern only sends new values
    std::vector<int> pat_ptr, pat_col;
    lina_gpu_ilu* ilu = nullptr;      // ILU(0) of M for RN_GPU_BICGSTAB_ILU
    bool ilu_stale = false;           // M has new values the factors do not reflect yet
    double f_old = 0;                 // functional at the start of the step

    double* vec() {
        double* p = lina::dev::alloc(n);
        owned.push_back(p);
        return p;
    }
    bool init(int dim) {
        n = dim;
        X = vec(), Xold = vec(), G = vec(), D = vec(), J = vec(), V1 = vec(), V2 = vec();
        B = vec(), S = vec(), T = vec(), T2 = vec(), rhs = vec(), lin = vec();
        for (double* p : owned)
            if (!p) return false;
        hX.resize(n), hG.resize(n), hD.resize(n), hJ.resize(n), hA.resize(n), hB.resize(n);
        return true;
    }
    void drop_row_list() {
        if (Mrow) free_sparse(Mrow);
        Mrow = nullptr;
    }
    void drop_M() {
        if (Mdev) lina_gpu_matrix_destroy(Mdev);
        Mdev = nullptr;
        if (ilu) lina_gpu_ilu_destroy(ilu);
        ilu = nullptr;
        ilu_stale = false;
        pat_ptr.clear();
        pat_col.clear();
        drop_row_list();
    }
    // M (host CSR in Mc) on the device: new values when the pattern is the last one, else a new matrix
    bool upload_M() {
        drop_row_list();
        if (Mdev && Mc.ptr == pat_ptr && Mc.col == pat_col) {
            if (lina_gpu_matrix_update_values(Mdev, Mc.val.data(), 0) != 0) return false;
            ilu_stale = ilu != nullptr;
            return true;
        }
        drop_M();
        if (lina_gpu_matrix_create(n, n, Mc.ptr.data(), Mc.col.data(), Mc.val.data(), &Mdev) != 0) return false;
        pat_ptr = Mc.ptr;
        pat_col = Mc.col;
        return true;
    }
    ~Ctx() {
        drop_M();
        for (double* p : owned) lina::dev::release(p);
        lina::dev::release(bounds.idx);
        lina::dev::release(bounds.lo);
        lina::dev::release(bounds.up);
    }
};

Ctx* g_ctx = nullptr;  // the call in progress (the reference's state is file-scope too)

// LINA_RN_TIMING set: seconds per phase of each Newton step on stderr (diagnostics)
struct PhaseClock {
    bool on = std::getenv("LINA_RN_TIMING") != nullptr;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    double lap() {
        if (!on) return 0.0;
        lina::dev::sync();
        auto now = std::chrono::steady_clock::now();
        double s = std::chrono::duration<double>(now - t).count();
        t = now;
        return s;
    }
};
double g_t_ilu = 0.0, g_t_krylov = 0.0;
int g_krylov_iters = 0;

// u . (A v) on the device
double bilinear(lina_gpu_matrix* A, const double* u, const double* v, double* tmp, int n) {
    lina::dev::sync();
    if (lina_gpu_matrix_spmv(A, LINA_PREC_FP64, v, tmp) != 0) return NAN;
    return lina::dev::dot(u, tmp, n);
}

// the functional at a device vector (RN_Functional, or x.H.x/2 + x.b on the GPU)
double functional(Ctx& c, const double* x) {
    if (rn_functional) {
        lina::dev::d2h(c.hX.data(), x, c.n);
        return rn_functional(c.hX.data(), c.n);
    }
    double q = bilinear(c.H, x, x, c.T2, c.n) / 2.;
    if (rn_b) q += lina::dev::dot(c.lin, x, c.n);
    return q;
}

// G = gradient at X (RN_gradient, or b + H x on the GPU)
bool gradient(Ctx& c) {
    if (rn_gradient) {
        lina::dev::d2h(c.hX.data(), c.X, c.n);
        double* g = rn_gradient(c.hX.data());
        if (!g) return false;
        bool ok = lina::dev::h2d(c.G, g, c.n);
        free(g);
        return ok;
    }
    lina::dev::sync();
    if (lina_gpu_matrix_spmv(c.H, LINA_PREC_FP64, c.X, c.G) != 0) return false;
    if (rn_b) lina::dev::axpy(c.G, 1., c.lin, c.n);
    return true;
}

// M = D H D + diag(|g| J) with the sparsity of the reference's two products
// (RN_get_M_D, reflective_newton.c:250-262: sparse_product of H with diag(D),
// then of diag(D) with that; zero factors skipped, zero results deleted)
void assemble_M(Ctx& c, const CsrCopy& H) {
    const int n = c.n;
    CsrCopy& M = c.Mc;
    M.n = n;
    M.ptr.assign(n + 1, 0);
    // row i of D H D kept entries (both factors and both products nonzero), then |g_i| J_i on the
    // diagonal; calls emit(k, v) in column order and returns the row's entry count
    auto row = [&](int i, auto emit) {
        int cnt = 0;
        const double di = c.hD[i];
        const double add = c.hJ[i] != 0.0 ? fabs(c.hG[i]) * c.hJ[i] : 0.0;
        bool diag_done = c.hJ[i] == 0.0;
        if (di != 0.0) {
            for (int p = H.ptr[i]; p < H.ptr[i + 1]; p++) {
                const int k = H.col[p];
                const double a = H.val[p], b = c.hD[k];
                if (a == 0.0 || b == 0.0) continue;
                const double hd = a * b;
                if (hd == 0.0) continue;
                const double v = di * hd;
                if (v == 0.0) continue;
                if (!diag_done && k >= i) {  // insert_sparse(M, |g_i| J_i, i, i)
                    if (k == i) {
                        emit(k, v + add);
                        cnt++;
                        diag_done = true;
                        continue;
                    }
                    emit(i, add);
                    cnt++;
                    diag_done = true;
                }
                emit(k, v);
                cnt++;
            }
        }
        if (cnt == 0 && diag_done) {  // the reference's (i, 0.0) of an empty row
            emit(i, 0.0);
            return 1;
        }
        if (!diag_done) {
            if (cnt == 0) {  // (i, 0.0) of the empty row, then the diagonal added to it
                emit(i, 0.0 + add);
                return 1;
            }
            emit(i, add);
            cnt++;
        }
        return cnt;
    };
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) M.ptr[i + 1] = row(i, [](int, double) {});
    for (int i = 0; i < n; i++) M.ptr[i + 1] += M.ptr[i];
    M.col.resize(M.ptr[n]);
    M.val.resize(M.ptr[n]);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        int q = M.ptr[i];
        row(i, [&](int k, double v) {
            M.col[q] = k;
            M.val[q] = v;
            q++;
        });
    }
}

}  // namespace

// ============================================================ step pieces
namespace {

double quadratic_on_circle(double x) {
    const double c = cos(x) * rn_Delta, s = sin(x) * rn_Delta;
    return c * (c * rn_ax + s * rn_axy + rn_bx) + s * (s * rn_ay + rn_by);
}

double rn_derivative(double x) {
    return ((sin(2. * x) * (-rn_ax + rn_ay) + cos(2. * x) * rn_axy) * rn_Delta - sin(x) * rn_bx + cos(x) * rn_by) *
           rn_Delta;
}

// minimum of the quadratic model on the circle of radius Delta in span(V1, V2)
// (subspace_minimum, reflective_newton.c:394-450); V1, V2 orthonormal; result in X
bool subspace_min_dev(lina_gpu_matrix* A, int n, const double* b, const double* V1, const double* V2, double* X,
                      double* tmp) {
    rn_bx = lina::dev::dot(V1, b, n);
    rn_by = lina::dev::dot(V2, b, n);
    rn_ax = bilinear(A, V1, V1, tmp, n);
    rn_ay = bilinear(A, V2, V2, tmp, n);
    rn_axy = bilinear(A, V1, V2, tmp, n) + bilinear(A, V2, V1, tmp, n);
    double* roots = nullptr;
    const int nroots = Interval_Separation_Newton_1D(rn_derivative, &roots, 0, 2. * M_PI, 500, 1e-6, 1000);
    if (nroots <= 0) {
        printf("subspace_minimum: no extrema found -> abort\n");
        free(roots);
        return false;
    }
    int m = 0;
    double best = quadratic_on_circle(roots[0]);
    for (int i = 1; i < nroots; i++)
        if (quadratic_on_circle(roots[i]) < best) {
            m = i;
            best = quadratic_on_circle(roots[i]);
        }
    lina::dev::d2d(X, V1, n);
    lina::dev::scal(X, rn_Delta * cos(roots[m]), n);
    lina::dev::axpy(X, rn_Delta * sin(roots[m]), V2, n);
    free(roots);
    return true;
}

// Largest-magnitude eigenpair by power iteration (power_method, linear_algebra.c:4802-4823): x <- A x (or
// (A - shift I) x), eigenvalue estimate x_new . x_old, x normalised, until the estimate changes by at most
// eps times the operator's mean absolute row sum (matrix_norm, :3441, of the shifted matrix for the
// shifted run).  prev is the estimate before the first step: the reference's second run starts from the
// caller's 0; its first run reads an unset value, for which at least two steps are taken here.
int power_iteration(lina_gpu_matrix* A, const CsrCopy& Ac, double shift, double* x, double* tmp, int n, int max_iter,
                    double eps, double prev0, bool two_steps, double* eig) {
    double q = 0;
    for (int i = 0; i < n; i++) {
        bool diag = false;
        for (int p = Ac.ptr[i]; p < Ac.ptr[i + 1]; p++) {
            if (Ac.col[p] == i) {
                diag = true;
                q += fabs(Ac.val[p] - shift);
            } else {
                q += fabs(Ac.val[p]);
            }
        }
        if (!diag && shift != 0) q += fabs(shift);
    }
    q /= n;
    double prev, lambda = prev0;
    int i = 0;
    double r;
    do {
        prev = lambda;
        lina::dev::sync();
        lina_gpu_matrix_spmv(A, LINA_PREC_FP64, x, tmp);
        if (shift != 0) lina::dev::axpy(tmp, -shift, x, n);
        lambda = lina::dev::dot(tmp, x, n);
        lina::dev::d2d(x, tmp, n);
        lina::dev::scal(x, 1. / sqrt(lina::dev::dot(x, x, n)), n);
        r = fabs(lambda - prev) / q;
        i++;
    } while ((r > eps || (two_steps && i == 1)) && i < max_iter);
    *eig = lambda;
    return i == max_iter ? 0 : i;
}

// set_random_normal_vector (linear_algebra.c:4823-4828): rand() / RAND_MAX after srand, normalised.  The
// reference seeds with time(NULL); the library seeds with kRnSeed so that runs repeat (the reference run
// with time() returning kRnSeed draws the same vector).
constexpr unsigned kRnSeed = 1;
void seeded_random_unit(double* x, int n, std::vector<double>& host) {
    srand(kRnSeed);
    for (int i = 0; i < n; i++) host[i] = (double)rand() / RAND_MAX;
    double nrm = 0;
    for (int i = 0; i < n; i++) nrm += host[i] * host[i];
    nrm = sqrt(nrm);
    for (int i = 0; i < n; i++) host[i] /= nrm;
    lina::dev::h2d(x, host.data(), n);
}

// RN_CHOLESKY (reflective_newton.c:332-338): the complete Cholesky factor C of M by cholesky_factorization
// (linear_algebra.c:2966-2983; dense, row by row, INDEFINITE when a diagonal square is negative), then
// L_triang_invert with C and U_triang_invert with C^T (:2008-2043) on v; the products of each row are
// subtracted in column order.  Dense: O(n^3) work and n^2 memory, as in the reference.
int cholesky_solve(const CsrCopy& M, int n, std::vector<double>& v) {
    std::vector<double> C((size_t)n * n, 0.0), A((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++)
        for (int p = M.ptr[i]; p < M.ptr[i + 1]; p++) A[(size_t)i * n + M.col[p]] = M.val[p];
    for (int i = 0; i < n; i++) {
        double* ci = &C[(size_t)i * n];
        for (int j = 0; j < i; j++) {
            const double* cj = &C[(size_t)j * n];
            double s = A[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= ci[k] * cj[k];
            ci[j] = s / cj[j];
        }
        double d = A[(size_t)i * n + i];
        for (int k = 0; k < i; k++) d -= ci[k] * ci[k];
        if (d < 0) return INDEFINITE;
        ci[i] = sqrt(d);
    }
    // forward: C y = v (rows of C in column order, the diagonal last)
    std::vector<double> b(v);
    double diag = 0;
    for (int i = 0; i < n; i++) {
        double sum = b[i];
        for (int j = 0; j <= i; j++) {
            const double c = C[(size_t)i * n + j];
            if (c == 0.0) continue;  // not stored in the reference's sparse factor
            if (j != i)
                sum -= c * v[j];
            else
                diag = c;
        }
        v[i] = sum / diag;
    }
    // backward: C^T x = y (row i of C^T holds C[j][i], j >= i, in column order)
    b = v;
    for (int i = n - 1; i >= 0; i--) {
        double sum = b[i];
        for (int j = i; j < n; j++) {
            const double c = C[(size_t)j * n + i];
            if (c == 0.0) continue;
            if (j != i)
                sum -= c * v[j];
            else
                diag = c;
        }
        v[i] = sum / diag;
    }
    return POSITIVE_DEFINITE;
}

sparse_matrix* row_list_M(Ctx& c) {
    if (!c.Mrow) c.Mrow = lina::api::from_csr(c.n, c.Mc.ptr.data(), c.Mc.col.data(), c.Mc.val.data());
    return c.Mrow;
}

// the local Newton solve M V2 = -D g and the fallback to negative curvature
// (RN_get_subspace, reflective_newton.c:294-392)
bool get_subspace(Ctx& c) {
    const int n = c.n;
    lina::dev::d2d(c.V1, c.G, n);
    lina::rn::pmult(c.V1, c.D, n);
    lina::dev::d2d(c.V2, c.V1, n);
    lina::dev::scal(c.V2, -1., n);
    lina::dev::d2d(c.rhs, c.V2, n);
    lina::dev::sync();
    int iter = 0;
    switch (rn_solver_type) {
        case RN_GPU_BICGSTAB_ILU: {
            // the factors of the last step's pattern are recomputed in place; a new pattern starts afresh
            PhaseClock pc;
            int frc = 0;
            if (!c.ilu)
                frc = lina_gpu_ilu_create_from_matrix(n, c.Mc.ptr.data(), c.Mc.col.data(), c.Mc.val.data(), &c.ilu);
            else if (c.ilu_stale)
                frc = lina_gpu_ilu_refactor(c.ilu, c.Mc.val.data(), 0);
            c.ilu_stale = false;
            if (frc != 0) {
                if (c.ilu) lina_gpu_ilu_destroy(c.ilu);
                c.ilu = nullptr;
                rn_status = INDEFINITE;
                break;
            }
            lina_gpu_solve_info info;
            g_t_ilu = pc.lap();
            lina_gpu_bicgstab(c.Mdev, c.ilu, LINA_PREC_MIXED, c.rhs, c.V2, lina::api::bi_eps_value(),
                              BI_get_max_iter(), LINA_PCG_DEVICE_PTRS | LINA_PCG_USE_X0, &info);
            g_t_krylov = pc.lap();
            g_krylov_iters = info.iterations;
            iter = info.iterations;
            rn_status = (info.status == 0 && iter < BI_get_max_iter()) ? POSITIVE_DEFINITE : INDEFINITE;
            break;
        }
        case RN_UMF:
        case RN_BICGSTAB:
        case RN_AMG:
        case RN_PCG: {
            sparse_matrix* M = row_list_M(c);
            RN_set_default_matrix(M);
            lina::dev::d2h(c.hA.data(), c.V2, n);
            lina::dev::d2h(c.hB.data(), c.rhs, n);
            if (rn_solver_type == RN_UMF) {
                rn_status = rn_local_solver ? rn_local_solver(M, c.hA.data(), c.hB.data()) : INDEFINITE;
            } else if (rn_solver_type == RN_BICGSTAB) {
                if (rn_amg) AMG_recompute_coarse_matrices(rn_amg, M);
                iter = BiCGStab_solve(c.hA.data(), c.hB.data(), n);
                rn_status = (iter >= 0 && iter < BI_get_max_iter()) ? POSITIVE_DEFINITE : INDEFINITE;
            } else if (rn_solver_type == RN_AMG) {
                if (rn_amg) AMG_recompute_coarse_matrices(rn_amg, M);
                iter = rn_amg ? AMG_solve(rn_amg, c.hB.data(), c.hA.data(), nullptr) : -1;
                rn_status = (iter >= 0 && iter < AMG_get_max_iter()) ? POSITIVE_DEFINITE : INDEFINITE;
            } else {
                sparse_matrix* L = sparse_zero(n);
                sparse_matrix* U = sparse_zero(n);
                rn_status = incomplete_LU_factorization(M, L, U);
                if (rn_status != INDEFINITE) {
                    PCG_default(M, L, U);
                    iter = pcg(c.hA.data(), c.hB.data(), n, rn_eps, rn_pcg_iter);
                    rn_status = (iter >= 0 && iter < rn_pcg_iter) ? POSITIVE_DEFINITE : INDEFINITE;
                }
                free_sparse(L);
                free_sparse(U);
            }
            lina::dev::h2d(c.V2, c.hA.data(), n);
            break;
        }
        case RN_CHOLESKY: {
            iter = 1;
            lina::dev::d2h(c.hA.data(), c.V2, n);
            rn_status = cholesky_solve(c.Mc, n, c.hA);
            if (rn_status != INDEFINITE) lina::dev::h2d(c.V2, c.hA.data(), n);
            break;
        }
        default:
            printf("Reflective Newton: local solver %d is not available in the GPU library\n", rn_solver_type);
            rn_status = INDEFINITE;
    }
    if (rn_status == INDEFINITE) {
        stats.number_neg_curv++;
        double shift = 0, curv = 0;
        // get_neg_curvature_direction (linear_algebra.c:4849-4866): the largest-magnitude eigenvalue, then
        // the shifted iteration from the same start vector towards the most negative curvature
        seeded_random_unit(c.V2, n, c.hA);
        power_iteration(c.Mdev, c.Mc, 0.0, c.V2, c.T, n, 1000, eig_eps, 0.0, true, &shift);
        seeded_random_unit(c.V2, n, c.hA);
        int it = power_iteration(c.Mdev, c.Mc, shift, c.V2, c.T, n, eig_iter, eig_eps, curv, false, &curv);
        curv += shift;
        stats.average_eig_iter += it;
        if (curv >= 0) {
            if (rn_info == YES) printf("Reflective Newton: not able to determine direction of negative curvature -> abort\n");
            if (kernel_dir) {
                lina::dev::h2d(c.V2, kernel_dir, n);
                lina::dev::scal(c.V2, 1. / sqrt(lina::dev::dot(c.V2, c.V2, n)), n);
            }
        } else if (rn_info == YES) {
            printf("\nnegative curvature: %f\nfound after %d iterations\n\n", curv, it);
        }
    }
    return true;
}

}  // namespace

// ============================================================ one step and the outer loop
namespace {

// sigma tests of the line search (RN_test_sigma_l/_u, reflective_newton.c:456-470); the curvature
// term uses the Hessian, not the scaled matrix
struct StepModel {
    double gs = 0, shs = 0;  // g.S and S.H.S
};

bool sigma_l(Ctx& c, const StepModel& m, double alpha) {
    const double dq = functional(c, c.X) - c.f_old;
    const double lower = rn_sigma_l * alpha * (m.gs + alpha * std::min(m.shs, 0.) / 2.);
    return dq < lower;
}

bool sigma_u(Ctx& c, const StepModel& m, double alpha) {
    const double dq = functional(c, c.X) - c.f_old;
    const double upper = rn_sigma_u * alpha * (m.gs + alpha * std::min(m.shs, 0.) / 2.);
    return dq > upper;
}

void step_to(Ctx& c, double alpha) {
    lina::dev::d2d(c.X, c.Xold, c.n);
    lina::dev::axpy(c.X, alpha, c.S, c.n);
    lina::rn::reflect(c.bounds, c.X);
}

// RN_iterate (reflective_newton.c:536-620)
bool iterate(Ctx& c) {
    const int n = c.n;
    const int max_ls = 10;
    lina::dev::d2d(c.Xold, c.X, n);
    c.f_old = functional(c, c.Xold);
    if (!get_subspace(c)) return false;
    lina::dev::d2d(c.B, c.G, n);
    lina::rn::pmult(c.B, c.D, n);
    const double bnorm = sqrt(lina::dev::dot(c.B, c.B, n));
    if (bnorm == 0) {
        if (rn_info == RN_YES) printf("contraction: %f\n", 1.);
        return true;
    }
    if (rn_status == POSITIVE_DEFINITE && sqrt(lina::dev::dot(c.V2, c.V2, n)) < rn_Delta) {
        lina::dev::d2d(c.S, c.V2, n);
    } else {
        lina::dev::scal(c.V1, 1. / sqrt(lina::dev::dot(c.V1, c.V1, n)), n);
        const double s = lina::dev::dot(c.V1, c.V2, n);
        lina::dev::axpy(c.V2, -s, c.V1, n);
        lina::dev::scal(c.V2, 1. / sqrt(lina::dev::dot(c.V2, c.V2, n)), n);
        if (!subspace_min_dev(c.Mdev, n, c.B, c.V1, c.V2, c.S, c.T)) return false;
    }
    lina::rn::pmult(c.S, c.D, n);
    StepModel m;
    m.gs = lina::dev::dot(c.G, c.S, n);
    m.shs = bilinear(c.H, c.S, c.S, c.T, n);
    double alpha = 1.0;
    step_to(c, alpha);
    if (!sigma_l(c, m, alpha)) {  // bisection line search
        stats.line_search_count++;
        int it = 0;
        double al = 0, ar = 1.;
        do {
            alpha = (al + ar) / 2.;
            step_to(c, alpha);
            if (!sigma_l(c, m, alpha)) {
                ar = alpha;
            } else {
                if (!sigma_u(c, m, alpha) && !(alpha > rn_rho))
                    al = alpha;
                else
                    break;
            }
            it++;
        } while (it < max_ls);
        if (rn_info == RN_YES && it == max_ls)
            printf("Reflective Newton warning: line search did not converge: alpha=%e\n", alpha);
        stats.line_search_iter += it;
    }
    if (lina::rn::at_boundary(c.bounds, c.X) == 1) {  // touched a bound: step back a little
        alpha -= rn_Xi * bnorm;
        step_to(c, alpha);
    }
    const double d = functional(c, c.X) - c.f_old;
    const double pred = m.gs + std::min(m.shs, 0.);
    const double contraction = d / pred;
    if (contraction > rn_trust_upper && d < 0) {
        rn_Delta = std::min(rn_trust_radius_max, 2. * rn_Delta);
        if (rn_info == RN_YES) printf("reflective Newton: increase trust radius: %e\n", rn_Delta);
    }
    if (contraction < rn_trust_lower || d >= 0) {
        rn_Delta = std::max(rn_trust_radius_min, rn_Delta / 2.);
        if (rn_info == RN_YES) printf("reflective Newton: decrease trust radius: %e\n", rn_Delta);
    }
    if (rn_info == RN_YES) printf("contraction: %f\n", contraction);
    return true;
}

bool upload_bounds(Ctx& c) {
    lina::rn::Bounds& b = c.bounds;
    b.nb = rn_bound_num;
    if (b.nb <= 0) return true;
    b.idx = (int*)lina::dev::alloc((b.nb + 1) / 2 + 1);  // FP64-sized allocation holding ints
    b.lo = lina::dev::alloc(b.nb);
    b.up = lina::dev::alloc(b.nb);
    if (!b.idx || !b.lo || !b.up) return false;
    return lina::dev::h2d_bytes(b.idx, rn_bound, (long)b.nb * sizeof(int)) && lina::dev::h2d(b.lo, rn_lower, b.nb) &&
           lina::dev::h2d(b.up, rn_upper, b.nb);
}

}  // namespace

extern "C" {

// reflective_newton (reflective_newton.c:660-711)
int reflective_newton(double* Xh) {
    if (rn_dim <= 0 || (!rn_hesse && !rn_compute_hesse)) {
        printf("Reflective Newton: no Hessian set -> abort\n");
        return -1;
    }
    Ctx c;
    if (!c.init(rn_dim) || !upload_bounds(c) || !lina::dev::h2d(c.X, Xh, c.n)) {
        fprintf(stderr, "LinA-GB300: reflective_newton: device allocation failed\n");
        return -1;
    }
    if (rn_b && !lina::dev::h2d(c.lin, rn_b, c.n)) return -1;
    const bool own_hesse = (rn_compute_hesse != nullptr);
    if (!own_hesse) c.H = lina::api::device_matrix(rn_hesse);
    std::vector<double> Q(rn_max_iter > 0 ? rn_max_iter : 1, 0.0);
    int iter = 0;
    double q = 0, dq = 0;
    double q0;
    if (own_hesse) {  // the default functional needs a Hessian before the first evaluation
        lina::dev::d2h(c.hX.data(), c.X, c.n);
        rn_hesse = rn_compute_hesse(c.hX.data());
        c.H = lina::api::device_matrix(rn_hesse);
    }
    q0 = functional(c, c.X);
    do {
        if (own_hesse && iter > 0) {
            lina::api::forget_device_matrix(rn_hesse);
            free_sparse(rn_hesse);
            lina::dev::d2h(c.hX.data(), c.X, c.n);
            rn_hesse = rn_compute_hesse(c.hX.data());
            c.H = lina::api::device_matrix(rn_hesse);
        }
        if (!c.H || !gradient(c)) return -1;
        lina::rn::set_DJ(c.n, c.bounds, c.G, c.X, c.D, c.J);
        lina::dev::d2h(c.hD.data(), c.D, c.n);
        lina::dev::d2h(c.hJ.data(), c.J, c.n);
        lina::dev::d2h(c.hG.data(), c.G, c.n);
        PhaseClock pc;
        if (own_hesse || iter == 0) c.Hc = lina::api::to_csr(rn_hesse);  // the Hessian changes only with a callback
        assemble_M(c, c.Hc);
        const double t_asm = pc.lap();
        if (!c.upload_M()) return -1;
        const double t_up = pc.lap();
        if (!iterate(c)) return -1;
        const double t_it = pc.lap();
        if (pc.on)
            fprintf(stderr, "RN step %d: assemble M %.3fs, upload %.3fs, step %.3fs (ILU set-up %.3fs, BiCGStab %.3fs "
                            "in %d iterations)\n",
                    iter, t_asm, t_up, t_it, g_t_ilu, g_t_krylov, g_krylov_iters);
        q = functional(c, c.X);
        dq = fabs((q - q0) / q0);
        if (iter < (int)Q.size()) Q[iter] = dq;
        if (rn_info == RN_YES) printf("overall reduction = %e\n\n", dq);
        iter++;
        q0 = q;
    } while (iter < rn_max_iter && dq > rn_eps);
    if (iter == rn_max_iter) printf("Reflective Newton: no convergence after %d iterations\n", iter);
    stats.res += dq;
    stats.total_iter += iter;
    stats.calls++;
    lina::rn::snap(c.bounds, c.X, 1e-3 * rn_eps);
    if (!lina::dev::d2h(Xh, c.X, c.n)) return -1;
    if (own_hesse && rn_hesse) {
        lina::api::forget_device_matrix(rn_hesse);
        free_sparse(rn_hesse);
        rn_hesse = nullptr;
    }
    if (rn_M == c.Mrow) rn_M = nullptr;
    return iter;
}

// subspace_minimum on host vectors (reflective_newton.c:394)
void subspace_minimum(sparse_matrix* A, double* b, double* V1, double* V2, double* X) {
    const int n = A->size;
    lina_gpu_matrix* m = lina::api::device_matrix(A);
    double *db = lina::dev::alloc(n), *d1 = lina::dev::alloc(n), *d2 = lina::dev::alloc(n), *dx = lina::dev::alloc(n),
           *dt = lina::dev::alloc(n);
    if (m && db && d1 && d2 && dx && dt && lina::dev::h2d(db, b, n) && lina::dev::h2d(d1, V1, n) &&
        lina::dev::h2d(d2, V2, n) && subspace_min_dev(m, n, db, d1, d2, dx, dt))
        lina::dev::d2h(X, dx, n);
    for (double* p : {db, d1, d2, dx, dt}) lina::dev::release(p);
}

}  // extern "C"

// ============================================================ CSR convenience entry point
extern "C" int lina_gpu_reflective_newton_csr(int n, const int* ptr, const int* col, const double* val,
                                              const double* b, const double* lower, const double* upper, double* x,
                                              int solver, int max_iter, double eps, double bi_eps) {
    if (n <= 0 || !ptr || !col || !val || !b || !lower || !upper || !x || max_iter < 1) {
        lina::dev::set_error("lina_gpu_reflective_newton_csr: invalid argument");
        return LINA_GPU_EINVAL;
    }
    sparse_matrix* H = lina::api::from_csr(n, ptr, col, val);
    std::vector<double> bb(b, b + n), lo(lower, lower + n), up(upper, upper + n);
    int* idx = get_all_indices(n);
    // the reference's defaults (reflective_newton.c:6-16) with the caller's limit and tolerance
    const int old_info = rn_info;
    RN_print_info(RN_NO);
    RN_set_params(max_iter, eps, 0.1, 0.9, 0.1, 250., 1., 0.6, 1.1, 1e-3, 1000.);
    set_RN_Hesse(H);
    set_RN_linear(bb.data());
    set_RN_functional(nullptr);
    RN_set_gradient(nullptr);
    set_RN_constraints(idx, lo.data(), up.data(), n);
    BI_set_eps(bi_eps);
    BI_set_max_iter(1000);
    RN_set_local_solver(nullptr);
    RN_set_solver(solver);
    const int it = reflective_newton(x);
    set_RN_Hesse(nullptr);
    set_RN_linear(nullptr);
    set_RN_constraints(nullptr, nullptr, nullptr, 0);
    RN_print_info(old_info);
    lina::api::forget_device_matrix(H);
    free_sparse(H);
    free(idx);
    return it;
}
