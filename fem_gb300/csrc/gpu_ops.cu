// gpu_ops.cu - device BLAS-1 for the LinA drop-in Krylov loops (see gpu_ops.h).
#include <cuda_runtime.h>

#include <cmath>

#include "gpu_ops.h"

namespace lina {
namespace dev {
namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 1024;

cudaStream_t g_stream = nullptr;
double* g_partials = nullptr;   // kBlocks partial sums
unsigned* g_ticket = nullptr;
double* g_result = nullptr;     // device scalar
double* g_host = nullptr;       // pinned host scalar

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// single-pass dot product: block partials, the last block sums them in index order
__global__ void __launch_bounds__(kThreads) dot_kernel(long n, const double* __restrict__ a,
                                                       const double* __restrict__ b, double* partials,
                                                       unsigned* ticket, double* out) {
    __shared__ double sm[32];
    __shared__ bool last;
    double v = 0.0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        v += a[i] * b[i];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double x = lane < nw ? sm[lane] : 0.0;
        x = warp_sum(x);
        if (lane == 0) partials[blockIdx.x] = x;
    }
    if (threadIdx.x == 0) {
        __threadfence();
        last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double x = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) x += __ldcg(partials + i);
    x = warp_sum(x);
    __syncthreads();
    if (lane == 0) sm[wid] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; w++) t += sm[w];
        *out = t;
        *ticket = 0u;
    }
}

__global__ void axpy_kernel(long n, double* __restrict__ y, double a, const double* __restrict__ x) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) y[i] += a * x[i];
}

__global__ void scal_kernel(long n, double* __restrict__ x, double a) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) x[i] *= a;
}

__global__ void xpay_kernel(long n, double* __restrict__ y, const double* __restrict__ x, double a) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        y[i] = x[i] + a * y[i];
}

int grid(long n) {
    long g = (n + kThreads - 1) / kThreads;
    if (g < 1) g = 1;
    if (g > kBlocks) g = kBlocks;
    return (int)g;
}

}  // namespace

bool ready() {
    if (g_stream) return true;
    if (cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking) != cudaSuccess) return false;
    if (cudaMalloc(&g_partials, kBlocks * sizeof(double)) != cudaSuccess) return false;
    if (cudaMalloc(&g_ticket, sizeof(unsigned)) != cudaSuccess) return false;
    if (cudaMalloc(&g_result, sizeof(double)) != cudaSuccess) return false;
    if (cudaMallocHost(&g_host, sizeof(double)) != cudaSuccess) return false;
    return cudaMemset(g_ticket, 0, sizeof(unsigned)) == cudaSuccess;
}

double* alloc(long n) {
    if (!ready()) return nullptr;
    void* p = nullptr;
    if (cudaMalloc(&p, (n > 0 ? n : 1) * sizeof(double)) != cudaSuccess) return nullptr;
    return (double*)p;
}

void release(void* p) {
    if (p) cudaFree(p);
}

bool h2d(double* d, const double* h, long n) {
    return cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, g_stream) == cudaSuccess &&
           cudaStreamSynchronize(g_stream) == cudaSuccess;
}

bool d2h(double* h, const double* d, long n) {
    return cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, g_stream) == cudaSuccess &&
           cudaStreamSynchronize(g_stream) == cudaSuccess;
}

bool d2d(double* d, const double* s, long n) {
    return cudaMemcpyAsync(d, s, n * sizeof(double), cudaMemcpyDeviceToDevice, g_stream) == cudaSuccess;
}

bool zero(double* d, long n) { return cudaMemsetAsync(d, 0, n * sizeof(double), g_stream) == cudaSuccess; }

double dot(const double* a, const double* b, long n) {
    dot_kernel<<<grid(n), kThreads, 0, g_stream>>>(n, a, b, g_partials, g_ticket, g_result);
    if (cudaMemcpyAsync(g_host, g_result, sizeof(double), cudaMemcpyDeviceToHost, g_stream) != cudaSuccess ||
        cudaStreamSynchronize(g_stream) != cudaSuccess)
        return NAN;
    return *g_host;
}

bool axpy(double* y, double a, const double* x, long n) {
    axpy_kernel<<<grid(n), kThreads, 0, g_stream>>>(n, y, a, x);
    return cudaGetLastError() == cudaSuccess;
}

bool scal(double* x, double a, long n) {
    scal_kernel<<<grid(n), kThreads, 0, g_stream>>>(n, x, a);
    return cudaGetLastError() == cudaSuccess;
}

bool xpay(double* y, const double* x, double a, long n) {
    xpay_kernel<<<grid(n), kThreads, 0, g_stream>>>(n, y, x, a);
    return cudaGetLastError() == cudaSuccess;
}

bool sync() { return cudaStreamSynchronize(g_stream) == cudaSuccess; }

void* stream() {
    ready();
    return (void*)g_stream;
}

}  // namespace dev
}  // namespace lina

#include "lina_gpu.h"

extern "C" int lina_gpu_dot(const double* a_dev, const double* b_dev, long n, double* result) {
    if (!a_dev || !b_dev || !result || n < 0) return LINA_GPU_EINVAL;
    if (!lina::dev::ready()) return LINA_GPU_ECUDA;
    double r = lina::dev::dot(a_dev, b_dev, n);
    if (std::isnan(r) && cudaGetLastError() != cudaSuccess) return LINA_GPU_ECUDA;
    *result = r;
    return 0;
}
