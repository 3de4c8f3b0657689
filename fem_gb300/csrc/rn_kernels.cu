// rn_kernels.cu - elementwise kernels of the reflective Newton step
// (LinA/reflective_newton.c): the scaling D and indicator J of the bound
// constraints (RN_set_D_J :227), the reflection into the box (RN_reflect :275),
// the final snap onto bounds (delete_small_diff :476) and the boundary test
// (is_at_boundary :498).  Constraint i acts on unknown idx[i] with bounds
// lo[i], up[i]; a NaN bound is absent.
#include <cuda_runtime.h>

#include <cmath>

#include "gpu_ops.h"
#include "rn_gpu.h"

namespace lina {
namespace rn {
namespace {

constexpr int kT = 256;

int grid(long n) {
    long g = (n + kT - 1) / kT;
    if (g < 1) g = 1;
    if (g > 4096) g = 4096;
    return (int)g;
}

cudaStream_t st() { return (cudaStream_t)lina::dev::stream(); }

__global__ void dj_init_kernel(long n, double* D, double* J) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        D[i] = 1.0;
        J[i] = 0.0;
    }
}

__global__ void dj_bound_kernel(int nb, const int* __restrict__ idx, const double* __restrict__ lo,
                                const double* __restrict__ up, const double* __restrict__ G,
                                const double* __restrict__ X, double* D, double* J) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const int k = idx[i];
        if (G[k] < 0) {
            if (!isnan(up[i])) {
                D[k] = sqrt(fabs(X[k] - up[i]));
                J[k] = 1.0;
            }
        } else {
            if (!isnan(lo[i])) {
                D[k] = sqrt(fabs(X[k] - lo[i]));
                J[k] = 1.0;
            }
        }
    }
}

__global__ void pmult_kernel(long n, double* a, const double* __restrict__ b) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) a[i] *= b[i];
}

__global__ void reflect_kernel(int nb, const int* __restrict__ idx, const double* __restrict__ lo,
                               const double* __restrict__ up, double* X) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const int k = idx[i];
        if (!isnan(lo[i])) {
            if (!isnan(up[i])) {
                const double d = 2. * (up[i] - lo[i]);
                double whole;
                const double w = modf(fabs(X[k] - lo[i]) / d, &whole) * d;
                X[k] = lo[i] + fmin(w, d - w);
            } else {
                X[k] = lo[i] + fabs(X[k] - lo[i]);
            }
        } else if (X[k] > up[i]) {
            X[k] = 2. * up[i] - X[k];
        }
    }
}

__global__ void snap_kernel(int nb, const int* __restrict__ idx, const double* __restrict__ lo,
                            const double* __restrict__ up, double* X, double eps) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const int k = idx[i];
        if (!isnan(up[i]) && fabs(X[k] - up[i]) < eps) X[k] = up[i];
        if (!isnan(lo[i]) && fabs(X[k] - lo[i]) < eps) X[k] = lo[i];
    }
}

__global__ void boundary_kernel(int nb, const int* __restrict__ idx, const double* __restrict__ lo,
                                const double* __restrict__ up, const double* __restrict__ X, int* flag) {
    const double eps = 1e-30;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const int k = idx[i];
        if ((!isnan(up[i]) && fabs(X[k] - up[i]) < eps) || (!isnan(lo[i]) && fabs(X[k] - lo[i]) < eps))
            *flag = 1;
    }
}

int* g_flag = nullptr;
int* g_flag_host = nullptr;

}  // namespace

bool set_DJ(long n, const Bounds& b, const double* G, const double* X, double* D, double* J) {
    dj_init_kernel<<<grid(n), kT, 0, st()>>>(n, D, J);
    if (b.nb > 0) dj_bound_kernel<<<grid(b.nb), kT, 0, st()>>>(b.nb, b.idx, b.lo, b.up, G, X, D, J);
    return cudaGetLastError() == cudaSuccess;
}

bool pmult(double* a, const double* b, long n) {
    pmult_kernel<<<grid(n), kT, 0, st()>>>(n, a, b);
    return cudaGetLastError() == cudaSuccess;
}

bool reflect(const Bounds& b, double* X) {
    if (b.nb > 0) reflect_kernel<<<grid(b.nb), kT, 0, st()>>>(b.nb, b.idx, b.lo, b.up, X);
    return cudaGetLastError() == cudaSuccess;
}

bool snap(const Bounds& b, double* X, double eps) {
    if (b.nb > 0) snap_kernel<<<grid(b.nb), kT, 0, st()>>>(b.nb, b.idx, b.lo, b.up, X, eps);
    return cudaGetLastError() == cudaSuccess;
}

int at_boundary(const Bounds& b, const double* X) {
    if (b.nb <= 0) return 0;
    if (!g_flag) {
        if (cudaMalloc(&g_flag, sizeof(int)) != cudaSuccess) return -1;
        if (cudaMallocHost(&g_flag_host, sizeof(int)) != cudaSuccess) return -1;
    }
    cudaMemsetAsync(g_flag, 0, sizeof(int), st());
    boundary_kernel<<<grid(b.nb), kT, 0, st()>>>(b.nb, b.idx, b.lo, b.up, X, g_flag);
    cudaMemcpyAsync(g_flag_host, g_flag, sizeof(int), cudaMemcpyDeviceToHost, st());
    if (cudaStreamSynchronize(st()) != cudaSuccess) return -1;
    return *g_flag_host;
}

}  // namespace rn
}  // namespace lina
