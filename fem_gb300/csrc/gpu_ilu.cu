// gpu_ilu.cu - ILU(0) preconditioner application on the GPU by level scheduling.
//
// The factors are the reference's (incomplete_LU_factorization,
// LinA/linear_algebra.c:1952-1982: L lower triangular with its diagonal, U
// upper triangular with a unit diagonal); applying the preconditioner is the
// forward solve L y = r followed by the backward solve U z = y
// (L_triang_invert / U_triang_invert, :2008-2043).  Rows are grouped into
// levels: a row's level is one more than the highest level among the rows it
// depends on, so all rows of a level can be solved at once.  On the structured
// meshes of this path the levels are anti-diagonals with a few hundred rows
// each, so one thread block walks all levels in order with a block barrier
// between levels: no inter-block waiting, no per-level launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "gpu_ops.h"
#include "lina_gpu.h"

namespace {

constexpr int kBlock = 1024;

template <typename TV, typename TX>
__global__ void __launch_bounds__(kBlock) tri_levels_kernel(int nlev, const int* __restrict__ lev_ptr,
                                                          const int* __restrict__ rows, const int* __restrict__ ptr,
                                                          const int* __restrict__ col, const TV* __restrict__ val,
                                                          const TX* __restrict__ dinv, const TX* __restrict__ b,
                                                          TX* x) {
    for (int l = 0; l < nlev; l++) {
        const int k1 = lev_ptr[l + 1];
        for (int k = lev_ptr[l] + threadIdx.x; k < k1; k += blockDim.x) {
            const int i = rows[k];
            TX s = b[i];
            for (int p = ptr[i]; p < ptr[i + 1]; p++) s -= TX(val[p]) * x[col[p]];
            x[i] = s * dinv[i];
        }
        __syncthreads();
    }
}

template <typename TA, typename TB>
__global__ void cvt_kernel(long n, const TA* __restrict__ a, TB* __restrict__ b) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = TB(a[i]);
}

struct Factor {
    int nlev = 0;
    std::vector<int> lev_ptr_h;
    int *lev_ptr = nullptr, *rows = nullptr, *ptr = nullptr, *col = nullptr;
    double *val64 = nullptr, *dinv64 = nullptr;
    float *val32 = nullptr, *dinv32 = nullptr;
};

template <typename T>
bool upload(T** d, const std::vector<T>& h) {
    size_t bytes = std::max<size_t>(1, h.size()) * sizeof(T);
    if (cudaMalloc((void**)d, bytes) != cudaSuccess) return false;
    return h.empty() || cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
}

// off-diagonal CSR of a triangular factor plus its inverse diagonal and level schedule;
// lower = true: rows depend on smaller indices (forward), else on larger ones (backward)
bool build_factor(Factor& f, int n, const int* p, const int* c, const double* v, bool lower, std::string& err) {
    std::vector<int> ptr(n + 1, 0), col;
    std::vector<double> val, dinv(n, 0.0);
    col.reserve(p[n]);
    val.reserve(p[n]);
    for (int i = 0; i < n; i++) {
        double d = 0.0;
        for (int k = p[i]; k < p[i + 1]; k++) {
            if (c[k] == i) {
                d = v[k];
            } else {
                if ((lower && c[k] > i) || (!lower && c[k] < i)) {
                    err = "factor is not triangular";
                    return false;
                }
                col.push_back(c[k]);
                val.push_back(v[k]);
            }
        }
        if (d == 0.0) {
            err = "zero diagonal in a triangular factor";
            return false;
        }
        dinv[i] = 1.0 / d;
        ptr[i + 1] = (int)col.size();
    }
    std::vector<int> lev(n, 0);
    int nlev = 0;
    for (int t = 0; t < n; t++) {
        const int i = lower ? t : n - 1 - t;
        int l = 0;
        for (int k = ptr[i]; k < ptr[i + 1]; k++) l = std::max(l, lev[col[k]] + 1);
        lev[i] = l;
        nlev = std::max(nlev, l + 1);
    }
    std::vector<int> lp(nlev + 1, 0), rows(n);
    for (int i = 0; i < n; i++) lp[lev[i] + 1]++;
    for (int l = 0; l < nlev; l++) lp[l + 1] += lp[l];
    std::vector<int> fill(lp.begin(), lp.end() - 1);
    for (int i = 0; i < n; i++) rows[fill[lev[i]]++] = i;
    std::vector<float> val32(val.begin(), val.end()), dinv32(dinv.begin(), dinv.end());
    f.nlev = nlev;
    f.lev_ptr_h = lp;
    bool ok = upload(&f.lev_ptr, lp) && upload(&f.rows, rows) && upload(&f.ptr, ptr) && upload(&f.col, col) &&
              upload(&f.val64, val) && upload(&f.dinv64, dinv) && upload(&f.val32, val32) &&
              upload(&f.dinv32, dinv32);
    if (!ok) err = "device allocation for the ILU factors failed";
    return ok;
}

void free_factor(Factor& f) {
    for (void* p : {(void*)f.lev_ptr, (void*)f.rows, (void*)f.ptr, (void*)f.col, (void*)f.val64, (void*)f.dinv64,
                    (void*)f.val32, (void*)f.dinv32})
        if (p) cudaFree(p);
    f = Factor();
}

std::string g_ilu_err;

}  // namespace

struct lina_gpu_ilu {
    int n = 0;
    Factor L, U;
    double* t64 = nullptr;
    float *r32 = nullptr, *t32 = nullptr, *z32 = nullptr;
};

extern "C" {

int lina_gpu_ilu_create(int n, const int* Lptr, const int* Lcol, const double* Lval, const int* Uptr,
                        const int* Ucol, const double* Uval, lina_gpu_ilu** out) {
    if (!out || n <= 0 || !Lptr || !Lcol || !Lval || !Uptr || !Ucol || !Uval) return LINA_GPU_EINVAL;
    *out = nullptr;
    lina_gpu_ilu* h = new lina_gpu_ilu();
    h->n = n;
    std::string err;
    if (!build_factor(h->L, n, Lptr, Lcol, Lval, true, err) || !build_factor(h->U, n, Uptr, Ucol, Uval, false, err) ||
        cudaMalloc(&h->t64, n * sizeof(double)) != cudaSuccess || cudaMalloc(&h->r32, n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&h->t32, n * sizeof(float)) != cudaSuccess || cudaMalloc(&h->z32, n * sizeof(float)) != cudaSuccess) {
        g_ilu_err = err.empty() ? "device allocation failed" : err;
        lina_gpu_ilu_destroy(h);
        return LINA_GPU_EINVAL;
    }
    *out = h;
    return 0;
}

int lina_gpu_ilu_destroy(lina_gpu_ilu* h) {
    if (!h) return 0;
    free_factor(h->L);
    free_factor(h->U);
    for (void* p : {(void*)h->t64, (void*)h->r32, (void*)h->t32, (void*)h->z32})
        if (p) cudaFree(p);
    delete h;
    return 0;
}

int lina_gpu_ilu_levels(const lina_gpu_ilu* h, int* nlev_L, int* nlev_U) {
    if (!h) return LINA_GPU_EINVAL;
    if (nlev_L) *nlev_L = h->L.nlev;
    if (nlev_U) *nlev_U = h->U.nlev;
    return 0;
}

// z = U^-1 L^-1 r on device vectors (FP64); precision LINA_PREC_MIXED runs both solves in FP32.
// The work is issued on the stream of the device vector toolkit and completes before return.
int lina_gpu_ilu_apply(lina_gpu_ilu* h, int precision, const double* r_dev, double* z_dev) {
    if (!h || !r_dev || !z_dev) return LINA_GPU_EINVAL;
    cudaStream_t st = (cudaStream_t)lina::dev::stream();
    const int n = h->n;
    const int g = (int)std::min<long>(2048, (n + 255) / 256);
    if (precision == LINA_PREC_MIXED) {
        cvt_kernel<double, float><<<g, 256, 0, st>>>(n, r_dev, h->r32);
        tri_levels_kernel<float, float><<<1, kBlock, 0, st>>>(h->L.nlev, h->L.lev_ptr, h->L.rows, h->L.ptr, h->L.col,
                                                              h->L.val32, h->L.dinv32, h->r32, h->t32);
        tri_levels_kernel<float, float><<<1, kBlock, 0, st>>>(h->U.nlev, h->U.lev_ptr, h->U.rows, h->U.ptr, h->U.col,
                                                              h->U.val32, h->U.dinv32, h->t32, h->z32);
        cvt_kernel<float, double><<<g, 256, 0, st>>>(n, h->z32, z_dev);
    } else {
        tri_levels_kernel<double, double><<<1, kBlock, 0, st>>>(h->L.nlev, h->L.lev_ptr, h->L.rows, h->L.ptr,
                                                                h->L.col, h->L.val64, h->L.dinv64, r_dev, h->t64);
        tri_levels_kernel<double, double><<<1, kBlock, 0, st>>>(h->U.nlev, h->U.lev_ptr, h->U.rows, h->U.ptr,
                                                                h->U.col, h->U.val64, h->U.dinv64, h->t64, z_dev);
    }
    if (cudaGetLastError() != cudaSuccess) return LINA_GPU_ECUDA;
    return cudaStreamSynchronize(st) == cudaSuccess ? 0 : LINA_GPU_ECUDA;
}

}  // extern "C"
