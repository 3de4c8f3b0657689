// gpu_gmres.cu - restarted GMRES on device vectors.
//
// Solves M y = b with M = B_l A B_r from an initial y, as the GMRES entry point
// of LinA does (LinA/gmres.c:308-500, the ZIB NewtonLib code): classical
// Gram-Schmidt Arnoldi (one pass), restart after i_max steps, the residual
// quotient eta = ||b - M y|| / ||b - M y_0|| tested at every step
// (CheckEachIter: y and the true residual are formed each step) or only at
// restarts, the step limit tested at restarts.  The small least-squares
// problem is solved on the host with Givens rotations (Saad, Iterative
// Methods for Sparse Linear Systems, 2nd ed., sec. 6.5.3).
//
// Device work per Arnoldi step: the operator (callbacks), one multi-dot
// kernel h_l = V_l . r for all l at once (r read once per chunk of eight
// basis vectors), one kernel forming v = r - sum_l h_l V_l together with
// |v|^2, and the normalisation; the host reads h and |v|^2 once per step.
// All reductions are single-pass and deterministic (block partials summed in
// a fixed order by the last block to finish).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "gmres_gpu.h"
#include "gpu_ops.h"
#include "lina_gpu.h"

namespace lina {
namespace gm {
namespace {

constexpr int kT = 256;
constexpr int kChunk = 8;
constexpr int kMaxGrid = 152 * 4;

cudaStream_t st() { return (cudaStream_t)lina::dev::stream(); }

int grid_for(long n) {
    long g = (n + kT - 1) / kT;
    return (int)std::max(1L, std::min(g, (long)kMaxGrid));
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block sum of v in a fixed order; the result is valid in thread 0
__device__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (warp == 0) {
        s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        s = warp_sum(s);
    }
    __syncthreads();
    return s;
}

// the last block to arrive sums the k rows of partials[k][gridDim.x] into out[k]
__device__ void finish_rows(int k, const double* partials, unsigned* ticket, double* out, double* sh) {
    __shared__ bool last;
    __threadfence();
    if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int l = 0; l < k; l++) {
        double s = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += partials[(long)l * gridDim.x + b];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) out[l] = s;
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

// out[l] = V_l . r, l < k
__global__ void mdot_kernel(long n, int k, const double* __restrict__ V, long ld, const double* __restrict__ r,
                            double* partials, unsigned* ticket, double* out) {
    __shared__ double sh[32];
    for (int l0 = 0; l0 < k; l0 += kChunk) {
        const int kc = min(kChunk, k - l0);
        double acc[kChunk];
#pragma unroll
        for (int j = 0; j < kChunk; j++) acc[j] = 0.0;
        for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
            const double rv = r[i];
#pragma unroll
            for (int j = 0; j < kChunk; j++)
                if (j < kc) acc[j] += V[(long)(l0 + j) * ld + i] * rv;
        }
        for (int j = 0; j < kc; j++) {
            const double s = block_sum(acc[j], sh);
            if (threadIdx.x == 0) partials[(long)(l0 + j) * gridDim.x + blockIdx.x] = s;
        }
    }
    finish_rows(k, partials, ticket, out, sh);
}

// w = r - sum_{l<k} h_l V_l and out = |w|^2
__global__ void orth_kernel(long n, int k, const double* __restrict__ V, long ld, const double* __restrict__ h,
                            const double* __restrict__ r, double* __restrict__ w, double* partials, unsigned* ticket,
                            double* out) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int l = 0; l < k; l++) s += V[(long)l * ld + i] * h[l];
        const double v = r[i] - s;
        w[i] = v;
        acc += v * v;
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    finish_rows(1, partials, ticket, out, sh);
}

// v = v / sqrt(*norm2)
__global__ void normalise_kernel(long n, double* __restrict__ v, const double* __restrict__ norm2) {
    const double nrm = sqrt(*norm2);
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        v[i] = v[i] / nrm;
}

// v = r / beta
__global__ void div_kernel(long n, double* __restrict__ v, const double* __restrict__ r, double beta) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        v[i] = r[i] / beta;
}

// y = y0 + sum_{l<k} z_l V_l
__global__ void combine_kernel(long n, int k, const double* __restrict__ V, long ld, const double* __restrict__ z,
                               const double* __restrict__ y0, double* __restrict__ y) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int l = 0; l < k; l++) s += V[(long)l * ld + i] * z[l];
        y[i] = y0[i] + s;
    }
}

// r = b - t and out = |r|^2
__global__ void resid_kernel(long n, const double* __restrict__ b, const double* __restrict__ t, double* __restrict__ r,
                             double* partials, unsigned* ticket, double* out) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double v = b[i] - t[i];
        r[i] = v;
        acc += v * v;
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    finish_rows(1, partials, ticket, out, sh);
}

// Givens rotation (c, s) with c a + s b = rho, -s a + c b = 0
void givens(double a, double b, double* c, double* s) {
    if (b == 0.0) {
        *c = 1.0;
        *s = 0.0;
    } else if (std::fabs(b) >= std::fabs(a)) {
        const double t = a / b;
        *s = 1.0 / std::sqrt(1.0 + t * t);
        *c = *s * t;
    } else {
        const double t = b / a;
        *c = 1.0 / std::sqrt(1.0 + t * t);
        *s = *c * t;
    }
}

struct Work {
    long n = 0;
    int kmax = 0;
    double* V = nullptr;  // (i_max + 2) basis vectors of length n
    double *r = nullptr, *w = nullptr, *y0 = nullptr, *t = nullptr;
    double* partials = nullptr;
    unsigned* ticket = nullptr;
    double* small = nullptr;  // device: h[kmax], norm2, z[kmax]
    double* host = nullptr;   // pinned mirror of small
    bool ok = false;
    Work(long n_, int i_max) : n(n_), kmax(i_max + 2) {
        ok = cudaMalloc(&V, sizeof(double) * n * kmax) == cudaSuccess &&
             cudaMalloc(&partials, sizeof(double) * (long)kMaxGrid * kmax) == cudaSuccess &&
             cudaMalloc(&ticket, sizeof(unsigned)) == cudaSuccess &&
             cudaMalloc(&small, sizeof(double) * (2 * kmax + 2)) == cudaSuccess &&
             cudaMallocHost(&host, sizeof(double) * (2 * kmax + 2)) == cudaSuccess;
        r = lina::dev::alloc(n), w = lina::dev::alloc(n), y0 = lina::dev::alloc(n), t = lina::dev::alloc(n);
        // the basis starts zeroed: a preconditioner that warm-starts from its output argument (the
        // AMG ones do) sees the same initial contents as with the reference's zeroed allocation
        ok = ok && r && w && y0 && t && cudaMemsetAsync(ticket, 0, sizeof(unsigned), st()) == cudaSuccess &&
             cudaMemsetAsync(V, 0, sizeof(double) * n * kmax, st()) == cudaSuccess;
    }
    ~Work() {
        cudaStreamSynchronize(st());
        if (V) cudaFree(V);
        if (partials) cudaFree(partials);
        if (ticket) cudaFree(ticket);
        if (small) cudaFree(small);
        if (host) cudaFreeHost(host);
        lina::dev::release(r);
        lina::dev::release(w);
        lina::dev::release(y0);
        lina::dev::release(t);
    }
    double* vec(int l) { return V + (long)l * n; }
};

}  // namespace

bool solve(long n, double* y, const double* b, const Op& matvec, const Op& preconr, const Op& preconl, double tol,
           int i_max, int max_iter, bool check_each, Result& res) {
    res = Result();
    Work W(n, i_max);
    if (!W.ok) {
        lina::dev::set_error("GMRES: device allocation failed");
        return false;
    }
    const int g = grid_for(n);
    double* d_h = W.small;
    double* d_norm = W.small + W.kmax;
    double* d_z = W.small + W.kmax + 1;
    // t = M x (x is left untouched; tmp receives B_r x)
    auto apply_M = [&](const double* x, double* tmp, double* out) -> bool {
        const double* xr = x;
        if (preconr) {
            if (!preconr(x, tmp)) return false;
            xr = tmp;
        }
        res.noprecr++;
        if (!preconl) {
            if (!matvec(xr, out)) return false;
        } else {
            if (!matvec(xr, W.w) || !preconl(W.w, out)) return false;
        }
        res.nomatvec++;
        res.noprecl++;
        return true;
    };
    auto residual = [&](const double* x, double* tmp, double* beta) -> bool {
        if (!apply_M(x, tmp, W.t)) return false;
        resid_kernel<<<g, kT, 0, st()>>>(n, b, W.t, W.r, W.partials, W.ticket, d_norm);
        if (cudaMemcpyAsync(W.host + W.kmax, d_norm, sizeof(double), cudaMemcpyDeviceToHost, st()) != cudaSuccess ||
            cudaStreamSynchronize(st()) != cudaSuccess)
            return false;
        *beta = std::sqrt(W.host[W.kmax]);
        return true;
    };
    std::vector<double> H((size_t)(i_max + 1) * (i_max + 1), 0.0);  // column j: H[j*(i_max+1) + l]
    std::vector<double> cs(i_max + 1), sn(i_max + 1), gvec(i_max + 2), z(i_max + 1);
    double beta0 = 0.0, beta1 = 0.0, eta = 0.0;
    int iter = 0;
    for (;;) {  // restart
        if (!lina::dev::d2d(W.y0, y, n)) return false;
        double beta;
        if (!residual(y, W.vec(0), &beta)) return false;
        if (iter == 0) {
            beta0 = beta;
            eta = (beta0 == 0.0) ? 0.0 : 1.0;
        } else {
            eta = beta / beta0;
        }
        beta1 = beta;
        if (beta > 0.0) div_kernel<<<g, kT, 0, st()>>>(n, W.vec(0), W.r, beta);
        std::fill(gvec.begin(), gvec.end(), 0.0);
        gvec[0] = beta;
        for (int i = 1; i <= i_max && eta > tol; i++) {
            // Arnoldi: r = M v_{i-1}; h_l = v_l . r; v_i = (r - sum h_l v_l) / |...|
            if (!apply_M(W.vec(i - 1), W.vec(i), W.r)) return false;
            mdot_kernel<<<g, kT, 0, st()>>>(n, i, W.V, n, W.r, W.partials, W.ticket, d_h);
            orth_kernel<<<g, kT, 0, st()>>>(n, i, W.V, n, d_h, W.r, W.vec(i), W.partials, W.ticket, d_norm);
            normalise_kernel<<<g, kT, 0, st()>>>(n, W.vec(i), d_norm);
            if (cudaGetLastError() != cudaSuccess ||
                cudaMemcpyAsync(W.host, W.small, sizeof(double) * (W.kmax + 1), cudaMemcpyDeviceToHost, st()) !=
                    cudaSuccess ||
                cudaStreamSynchronize(st()) != cudaSuccess) {
                lina::dev::set_error("GMRES: device step failed");
                return false;
            }
            const double normv = std::sqrt(W.host[W.kmax]);
            // new Hessenberg column, rotated by the previous rotations
            double* col = &H[(size_t)(i - 1) * (i_max + 1)];
            for (int l = 0; l < i; l++) col[l] = W.host[l];
            double sub = normv;
            for (int l = 0; l < i - 1; l++) {
                const double a = col[l], bb = col[l + 1];
                col[l] = cs[l] * a + sn[l] * bb;
                col[l + 1] = -sn[l] * a + cs[l] * bb;
            }
            givens(col[i - 1], sub, &cs[i - 1], &sn[i - 1]);
            col[i - 1] = cs[i - 1] * col[i - 1] + sn[i - 1] * sub;
            gvec[i] = -sn[i - 1] * gvec[i - 1];
            gvec[i - 1] = cs[i - 1] * gvec[i - 1];
            if (col[i - 1] == 0.0) {  // singular Hessenberg system
                res.rcode = 1;
                res.iter = iter;
                res.precision = eta;
                return true;
            }
            const bool breakdown = (normv == 0.0);
            if (check_each || i == i_max || breakdown) {
                for (int l = i - 1; l >= 0; l--) {  // back substitution
                    double s = gvec[l];
                    for (int m = l + 1; m < i; m++) s -= H[(size_t)m * (i_max + 1) + l] * z[m];
                    z[l] = s / H[(size_t)l * (i_max + 1) + l];
                }
                if (cudaMemcpyAsync(d_z, z.data(), sizeof(double) * i, cudaMemcpyHostToDevice, st()) != cudaSuccess)
                    return false;
                combine_kernel<<<g, kT, 0, st()>>>(n, i, W.V, n, d_z, W.y0, y);
                if (check_each) {
                    if (!residual(y, W.vec(i + 1), &beta1)) return false;
                    eta = beta1 / beta0;
                }
            }
            iter++;
            if (breakdown) break;  // the Krylov space is invariant: y solves the system
        }
        if (eta > tol && iter < max_iter) continue;
        res.rcode = (eta <= tol) ? 0 : 2;
        break;
    }
    if (!lina::dev::sync()) return false;
    res.iter = iter;
    res.precision = eta;
    res.residuum = beta1;
    return true;
}

}  // namespace gm
}  // namespace lina

// ---------------------------------------------------------------- C-ABI
extern "C" int lina_gpu_gmres(lina_gpu_matrix* A, lina_gpu_ilu* ilu, lina_gpu_amg* amg, int precon_precision,
                              const double* b, double* y, double tol, int i_max, int max_iter, int check_each_iter,
                              int flags, lina_gpu_solve_info* info) {
    if (!A || !b || !y || (ilu && amg) || i_max < 1 || max_iter < 1 || !(tol > 0)) {
        lina::dev::set_error("lina_gpu_gmres: invalid argument");
        return LINA_GPU_EINVAL;
    }
    const long n = lina_gpu_matrix_rows(A);
    const bool dev = (flags & LINA_PCG_DEVICE_PTRS) != 0;
    double* db = nullptr;
    double* dy = nullptr;
    double* tmp = nullptr;
    auto cleanup = [&]() {
        if (!dev) {
            lina::dev::release(db);
            lina::dev::release(dy);
        }
        lina::dev::release(tmp);
    };
    if (dev) {
        db = const_cast<double*>(b);
        dy = y;
    } else {
        db = lina::dev::alloc(n);
        dy = lina::dev::alloc(n);
        if (!db || !dy || !lina::dev::h2d(db, b, n) || !lina::dev::h2d(dy, y, n)) {
            cleanup();
            return LINA_GPU_ECUDA;
        }
    }
    lina::gm::Op matvec = [&](const double* x, double* out) {
        lina::dev::sync();
        return lina_gpu_matrix_spmv(A, LINA_PREC_FP64, x, out) == 0;
    };
    lina::gm::Op preconr;
    if (ilu)
        preconr = [&](const double* x, double* out) {
            lina::dev::sync();
            return lina_gpu_ilu_apply(ilu, precon_precision, x, out) == 0;
        };
    else if (amg)
        preconr = [&](const double* x, double* out) {
            lina::dev::sync();
            return lina_gpu_vcycle(amg, x, out) == 0;
        };
    lina::gm::Result r;
    const bool ok = lina::gm::solve(n, dy, db, matvec, preconr, lina::gm::Op(), tol, i_max, max_iter,
                                    check_each_iter != 0, r);
    int rc = ok ? 0 : LINA_GPU_ECUDA;
    if (ok && (flags & LINA_GMRES_APPLY_PRECON) && preconr) {  // x = B_r y
        tmp = lina::dev::alloc(n);
        if (!tmp || !preconr(dy, tmp) || !lina::dev::d2d(dy, tmp, n)) rc = LINA_GPU_ECUDA;
    }
    if (rc == 0 && !dev && !lina::dev::d2h(y, dy, n)) rc = LINA_GPU_ECUDA;
    if (info) {
        info->iterations = r.iter;
        info->rel_residual = r.precision;
        info->status = rc ? rc : (r.rcode == 0 ? 0 : (r.rcode == 2 ? LINA_GPU_ENOCONV : LINA_GPU_EBREAKDOWN));
        info->true_rel_residual = NAN;
        info->pcg_residuum = NAN;
        info->smoother_ms = 0;
        info->smoother_launches = 0;
        info->smoother_bytes = 0;
        info->timed_level = 0;
        info->timed_rows = 0;
        info->timed_entries = 0;
    }
    cleanup();
    if (rc) return rc;
    return r.rcode == 0 ? 0 : (r.rcode == 2 ? LINA_GPU_ENOCONV : LINA_GPU_EBREAKDOWN);
}
