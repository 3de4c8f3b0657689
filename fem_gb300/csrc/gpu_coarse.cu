// gpu_coarse.cu - the coarsest AMG level's dense block inverted on the GPU.
//
// The reference factorises the block of coarsest rows holding more than one nonzero with a dense LU
// without pivoting (sparse_LU_factorization, LinA/linear_algebra.c:3040, LU_factorzation :2909) and
// solves with it in every V-cycle (AMG_Direct_solver, LinA/Multigrid.c:1450).  This library keeps the
// block's inverse so that the coarse solve is one dense matrix-vector product on the GPU; here the
// inverse is formed on the device, in place, by blocked Gauss-Jordan elimination without pivoting
// (the same elimination order as the reference's LU, so it exists exactly when the reference's
// factorisation does).  For a pivot block K of 32 rows, with I, J the other rows and columns:
//     A_KK <- A_KK^-1,  A_KJ <- A_KK^-1 A_KJ,  A_IJ <- A_IJ - A_IK A_KJ,  A_IK <- -A_IK A_KK^-1
// The rank-32 update of A_IJ is 2 m^2 32 flops per step, 2 m^3 in total: it runs either on the FP64
// CUDA cores (4 x 4 outputs per thread) or on the FP64 tensor cores (mma.sync m8n8k4 FP64, the DMMA
// instruction; tcgen05 has no FP64 kind).  lina_gpu_dense_inverse exposes both for measurement.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "lina_gpu.h"

namespace {

constexpr int kNb = 32;      // pivot block
constexpr int kTile = 64;    // output tile of the trailing update (rows x columns)

// the diagonal block inverted in place by unblocked Gauss-Jordan (one CTA, bs <= 32); err = 1 on a zero
// pivot
__global__ void __launch_bounds__(kNb * kNb) diag_inverse_kernel(int m, int k0, int bs, double* A, int* err) {
    __shared__ double D[kNb][kNb + 1];
    const int r = threadIdx.x / kNb, c = threadIdx.x % kNb;
    D[r][c] = (r < bs && c < bs) ? A[(size_t)(k0 + r) * m + k0 + c] : 0.0;
    __syncthreads();
    for (int p = 0; p < bs; p++) {
        const double piv = D[p][p];
        if (piv == 0.0) {
            if (threadIdx.x == 0) atomicExch(err, 1);
            return;  // uniform: every thread read the same pivot
        }
        const double ip = 1.0 / piv;
        const double dip = D[r][p];
        const double dpc = D[p][c];
        __syncthreads();
        if (r < bs && c < bs) {
            if (r == p && c == p)
                D[r][c] = ip;
            else if (r == p)
                D[r][c] = dpc * ip;
            else if (c == p)
                D[r][c] = -dip * ip;
            else
                D[r][c] = D[r][c] - dip * (dpc * ip);
        }
        __syncthreads();
    }
    if (r < bs && c < bs) A[(size_t)(k0 + r) * m + k0 + c] = D[r][c];
}

// A_KJ <- A_KK^-1 A_KJ for every column j outside K (one thread per column)
__global__ void row_panel_kernel(int m, int k0, int bs, double* A) {
    __shared__ double Di[kNb][kNb];
    for (int t = threadIdx.x; t < kNb * kNb; t += blockDim.x) {
        const int r = t / kNb, c = t % kNb;
        Di[r][c] = (r < bs && c < bs) ? A[(size_t)(k0 + r) * m + k0 + c] : 0.0;
    }
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m || (j >= k0 && j < k0 + bs)) return;
    double col[kNb];
#pragma unroll
    for (int r = 0; r < kNb; r++) col[r] = (r < bs) ? A[(size_t)(k0 + r) * m + j] : 0.0;
    for (int r = 0; r < bs; r++) {
        double s = 0.0;
#pragma unroll
        for (int c = 0; c < kNb; c++) s += Di[r][c] * col[c];
        A[(size_t)(k0 + r) * m + j] = s;
    }
}

// A_IK <- -A_IK A_KK^-1 for every row i outside K (one thread per row)
__global__ void col_panel_kernel(int m, int k0, int bs, double* A) {
    __shared__ double Di[kNb][kNb];
    for (int t = threadIdx.x; t < kNb * kNb; t += blockDim.x) {
        const int r = t / kNb, c = t % kNb;
        Di[r][c] = (r < bs && c < bs) ? A[(size_t)(k0 + r) * m + k0 + c] : 0.0;
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || (i >= k0 && i < k0 + bs)) return;
    double row[kNb];
#pragma unroll
    for (int c = 0; c < kNb; c++) row[c] = (c < bs) ? A[(size_t)i * m + k0 + c] : 0.0;
    for (int c = 0; c < bs; c++) {
        double s = 0.0;
#pragma unroll
        for (int r = 0; r < kNb; r++) s += row[r] * Di[r][c];
        A[(size_t)i * m + k0 + c] = -s;
    }
}

// the K panels of a 64 x 64 output tile, staged in shared memory: Cs = A[tile rows][K], Rs = A[K][tile cols]
__device__ __forceinline__ void stage_panels(int m, int k0, int bs, int i0, int j0, const double* A,
                                             double (*Cs)[kNb + 1], double (*Rs)[kTile + 1]) {
    for (int t = threadIdx.x; t < kTile * kNb; t += blockDim.x) {
        const int r = t / kNb, c = t % kNb;
        const int i = i0 + r;
        Cs[r][c] = (i < m && c < bs) ? A[(size_t)i * m + k0 + c] : 0.0;
    }
    for (int t = threadIdx.x; t < kNb * kTile; t += blockDim.x) {
        const int r = t / kTile, c = t % kTile;
        const int j = j0 + c;
        Rs[r][c] = (j < m && r < bs) ? A[(size_t)(k0 + r) * m + j] : 0.0;
    }
}

// A_IJ -= A_IK A_KJ on FP64 CUDA cores: 256 threads, 4 x 4 outputs each
__global__ void __launch_bounds__(256) update_simt_kernel(int m, int k0, int bs, double* A) {
    __shared__ double Cs[kTile][kNb + 1];
    __shared__ double Rs[kNb][kTile + 1];
    const int i0 = blockIdx.y * kTile, j0 = blockIdx.x * kTile;
    stage_panels(m, k0, bs, i0, j0, A, Cs, Rs);
    __syncthreads();
    const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
    double acc[4][4] = {};
    for (int k = 0; k < kNb; k++) {
        double a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; u++) a[u] = Cs[tr + 16 * u][k], b[u] = Rs[k][tc + 16 * u];
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) {
            const int i = i0 + tr + 16 * u, j = j0 + tc + 16 * v;
            if (i < m && j < m && !(i >= k0 && i < k0 + bs) && !(j >= k0 && j < k0 + bs))
                A[(size_t)i * m + j] -= acc[u][v];
        }
}

// A_IJ -= A_IK A_KJ on FP64 tensor cores: mma.sync.m8n8k4 FP64.  Eight warps in a 4 x 2 grid, each
// computing a 16 x 32 part of the 64 x 64 tile as 2 x 4 MMA tiles of 8 x 8 over K in steps of 4.
// Fragments (PTX ISA, m8n8k4 .f64): A (8 x 4, row-major) lane l holds A[l / 4][l % 4]; B (4 x 8,
// column-major) lane l holds B[l % 4][l / 4]; C and D (8 x 8) lane l holds C[l / 4][2 (l % 4) + {0, 1}].
__global__ void __launch_bounds__(256) update_dmma_kernel(int m, int k0, int bs, double* A) {
    __shared__ double Cs[kTile][kNb + 1];
    __shared__ double Rs[kNb][kTile + 1];
    const int i0 = blockIdx.y * kTile, j0 = blockIdx.x * kTile;
    stage_panels(m, k0, bs, i0, j0, A, Cs, Rs);
    __syncthreads();
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int wr = (warp / 2) * 16, wc = (warp % 2) * 32;
    double acc[2][4][2] = {};
    for (int k = 0; k < kNb; k += 4) {
        double a[2], b[4];
#pragma unroll
        for (int u = 0; u < 2; u++) a[u] = Cs[wr + 8 * u + lane / 4][k + lane % 4];
#pragma unroll
        for (int v = 0; v < 4; v++) b[v] = Rs[k + lane % 4][wc + 8 * v + lane / 4];
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
            for (int v = 0; v < 4; v++)
                asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                             : "+d"(acc[u][v][0]), "+d"(acc[u][v][1])
                             : "d"(a[u]), "d"(b[v]));
    }
#pragma unroll
    for (int u = 0; u < 2; u++)
#pragma unroll
        for (int v = 0; v < 4; v++)
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int i = i0 + wr + 8 * u + lane / 4, j = j0 + wc + 8 * v + 2 * (lane % 4) + e;
                if (i < m && j < m && !(i >= k0 && i < k0 + bs) && !(j >= k0 && j < k0 + bs))
                    A[(size_t)i * m + j] -= acc[u][v][e];
            }
}

thread_local std::string g_coarse_err;

}  // namespace

namespace lina {

// In-place inverse of the dense m x m row-major matrix a_dev on the device (stream st); method
// LINA_DENSE_SIMT or LINA_DENSE_DMMA.  Returns 0, LINA_GPU_ESETUP on a zero pivot (the block row in
// the message), LINA_GPU_ECUDA on a CUDA error.
int dense_inverse(int m, double* a_dev, int method, cudaStream_t st, int* err_dev, std::string& msg) {
    if (m <= 0) return 0;
    if (cudaMemsetAsync(err_dev, 0, sizeof(int), st) != cudaSuccess) {
        msg = "dense inverse: clearing the error word failed";
        return LINA_GPU_ECUDA;
    }
    const int tiles = (m + kTile - 1) / kTile;
    for (int k0 = 0; k0 < m; k0 += kNb) {
        const int bs = (m - k0 < kNb) ? m - k0 : kNb;
        diag_inverse_kernel<<<1, kNb * kNb, 0, st>>>(m, k0, bs, a_dev, err_dev);
        row_panel_kernel<<<(m + 127) / 128, 128, 0, st>>>(m, k0, bs, a_dev);
        if (method == LINA_DENSE_DMMA)
            update_dmma_kernel<<<dim3(tiles, tiles), 256, 0, st>>>(m, k0, bs, a_dev);
        else
            update_simt_kernel<<<dim3(tiles, tiles), 256, 0, st>>>(m, k0, bs, a_dev);
        col_panel_kernel<<<(m + 127) / 128, 128, 0, st>>>(m, k0, bs, a_dev);
    }
    int err = 0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&err, err_dev, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        msg = "dense inverse: CUDA error";
        return LINA_GPU_ECUDA;
    }
    if (err) {
        msg = "coarsest level: zero pivot in the dense block (no pivoting, as the reference's LU)";
        return LINA_GPU_ESETUP;
    }
    return 0;
}

}  // namespace lina

extern "C" int lina_gpu_dense_inverse(int m, double* a_dev, int method, double* ms) {
    if (m < 0 || (m > 0 && !a_dev) || (method != LINA_DENSE_SIMT && method != LINA_DENSE_DMMA)) {
        g_coarse_err = "lina_gpu_dense_inverse: invalid argument";
        return LINA_GPU_EINVAL;
    }
    int* err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return LINA_GPU_ECUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, 0);
    std::string msg;
    const int rc = lina::dense_inverse(m, a_dev, method, 0, err, msg);
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    if (ms) *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(err);
    if (rc) fprintf(stderr, "LinA-GB300: %s\n", msg.c_str());
    return rc;
}
