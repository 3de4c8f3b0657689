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

bool h2d_bytes(void* d, const void* h, long bytes) {
    return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, g_stream) == cudaSuccess &&
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

// ---------------------------------------------------------------- allocation-free dot product
// Some callers cannot allocate device memory where they need a reduction: an
// application that reserves the GPU's memory for its own pool when it starts
// (so a cudaMalloc in the middle of its time step fails or is forbidden), or a
// job that runs under a hard device-memory quota.  lina_gpu_dot computes the
// same product but obtains its partial-sum buffer from cudaMalloc on first
// use; lina_gpu_dot_noalloc keeps that scratch in a fixed array that the
// module itself defines in device memory, so the call allocates nothing.
//
// The array holds one partial sum per block of 2048 elements plus the result
// and an arrival counter: 16,384 partials, so at most 33,554,432 elements per
// call (larger n is rejected).  It is 128 KB and occupies every GPU that loads
// the library for as long as the process runs.  All calls share it and it
// keeps the last call's contents; the arrival counter is cleared before every
// launch.  Calls whose kernels overlap on the GPU (different streams, other
// threads) race on the shared array and give wrong results: issue them one at
// a time.
//
// The call is synchronous: it waits for the library's own stream (the drop-in
// BLAS-1 helpers may still be writing a or b there), runs on the legacy
// default stream, and copies the result to the host.  It therefore cannot be
// captured into a CUDA graph, and it may not be called from a host function
// enqueued on a stream (such functions may make no CUDA calls).  Vectors that
// the caller produced on its own non-blocking streams must be complete before
// the call: synchronize those streams first.
//
// The first call on each device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and keeps it for the life of
// the process.  Make that first call before any stream capture begins.  A
// cudaDeviceReset unloads the module and invalidates the kept address: do not
// use this entry point after the host application resets the device.
namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 8;
constexpr long kNoAllocPerBlock = (long)kNoAllocThreads * kNoAllocPerThread;  // 2048 elements
constexpr int kNoAllocMaxBlocks = 16384;
constexpr long kNoAllocMaxN = kNoAllocPerBlock * kNoAllocMaxBlocks;  // 33,554,432 elements
constexpr int kNoAllocResult = kNoAllocMaxBlocks;                     // slot of the result
constexpr int kNoAllocCounter = kNoAllocMaxBlocks + 1;                // slot holding the arrival counter
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_dot_scratch[kNoAllocMaxBlocks + 2];

double* g_dot_scratch_addr[kMaxDevices] = {nullptr};

__global__ void __launch_bounds__(kNoAllocThreads) dot_noalloc_kernel(long n, const double* __restrict__ a,
                                                                      const double* __restrict__ b,
                                                                      double* scratch) {
    __shared__ double sm[kNoAllocThreads / 32];
    __shared__ bool last;
    unsigned* counter = reinterpret_cast<unsigned*>(scratch + kNoAllocCounter);
    const long base = (long)blockIdx.x * kNoAllocPerBlock;
    double v = 0.0;
#pragma unroll
    for (int k = 0; k < kNoAllocPerThread; k++) {
        const long i = base + (long)k * kNoAllocThreads + threadIdx.x;
        if (i < n) v += a[i] * b[i];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = lina::dev::warp_sum(v);
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kNoAllocThreads / 32; w++) t += sm[w];
        scratch[blockIdx.x] = t;
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double x = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kNoAllocThreads) x += __ldcg(scratch + i);
    x = lina::dev::warp_sum(x);
    __syncthreads();
    if (lane == 0) sm[wid] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kNoAllocThreads / 32; w++) t += sm[w];
        scratch[kNoAllocResult] = t;
        *counter = 0u;
    }
}

}  // namespace

extern "C" int lina_gpu_dot_noalloc(const double* a_dev, const double* b_dev, long n, double* result) {
    if (!a_dev || !b_dev || !result || n < 0) {
        lina::dev::set_error("lina_gpu_dot_noalloc: null pointer or negative length");
        return LINA_GPU_EINVAL;
    }
    if (n > kNoAllocMaxN) {
        lina::dev::set_error("lina_gpu_dot_noalloc: n exceeds the allocation-free limit of 33554432 elements "
                             "(use lina_gpu_dot)");
        return LINA_GPU_EINVAL;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) {
        lina::dev::set_error("lina_gpu_dot_noalloc: no usable current device");
        return LINA_GPU_ECUDA;
    }
    if (!g_dot_scratch_addr[device]) {
        double* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&p, g_dot_scratch);
        if (e != cudaSuccess || !p) {
            lina::dev::set_error("lina_gpu_dot_noalloc: cudaGetSymbolAddress of the scratch array failed");
            return LINA_GPU_ECUDA;
        }
        g_dot_scratch_addr[device] = p;
    }
    double* scratch = g_dot_scratch_addr[device];
    if (n == 0) {
        *result = 0.0;
        return 0;
    }
    // the library's drop-in vector helpers run on its non-blocking stream, which the legacy default
    // stream does not wait for
    if (lina::dev::g_stream && cudaStreamSynchronize(lina::dev::g_stream) != cudaSuccess) {
        lina::dev::set_error("lina_gpu_dot_noalloc: waiting for the library's stream failed");
        return LINA_GPU_ECUDA;
    }
    if (cudaMemsetAsync(scratch + kNoAllocCounter, 0, sizeof(double), 0) != cudaSuccess) {
        lina::dev::set_error("lina_gpu_dot_noalloc: clearing the arrival counter failed");
        return LINA_GPU_ECUDA;
    }
    const int grid = (int)((n + kNoAllocPerBlock - 1) / kNoAllocPerBlock);
    dot_noalloc_kernel<<<grid, kNoAllocThreads, 0, 0>>>(n, a_dev, b_dev, scratch);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(result, scratch + kNoAllocResult, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
        lina::dev::set_error("lina_gpu_dot_noalloc: kernel or result copy failed");
        return LINA_GPU_ECUDA;
    }
    return 0;
}
