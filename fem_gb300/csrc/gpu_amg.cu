// gpu_amg.cu - sm_103a kernels and device-side driver of the AMG-preconditioned
// Krylov solve (the solve phase of LinA's AMG_solve / pcg on one GB300).
//
// Layout in HBM, per level: CSR with int32 row pointers and column indices and
// two value arrays (FP64 for the plain path, FP32 for the mixed-precision
// preconditioner), the inverse diagonal in both precisions, the rows of each
// colour class (multicolour SOR), and per-level work vectors.  The coarsest
// level is a dense FP64 inverse of its non-isolated block (one GEMV per
// V-cycle).  Every kernel is bandwidth-bound; the arithmetic is CUDA-core
// FP64/FP32.  Reductions are single-pass: each block writes one partial and the
// last block to finish (atomic ticket, no waiting) sums the partials in a fixed
// order, so results are bitwise reproducible from run to run.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <sys/stat.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "amg_host.h"
#include "gpu_ops.h"
#include "lina_gpu.h"

namespace lina {
int dense_inverse(int m, double* a_dev, int method, cudaStream_t st, int* err_dev, std::string& msg);
}

namespace {

std::string g_err;
unsigned long long g_launches = 0;  // kernels launched by this library (all handles)
int g_layout = 0;  // 0 automatic, 1 SELL-32, 2 lane groups (size chosen per matrix), 3..6 groups of 4..32 lanes
// levels of at most this many rows run a multicolour-SOR V-cycle step as one thread-block-cluster launch
// (0: one launch per colour and step).  Measured on the batch workload: up to 24,576 rows the fused
// steps win; at 49,152 the levels whose colours need several passes of the cluster's lane groups
// made whole solves up to 30 % slower.
int g_fused_rows = 24576;
// damped Jacobi: levels of at most this many stored entries (and g_fused_rows rows) run a V-cycle step as
// one cluster launch; off by default.  Measured on the 2.1M-dof elasticity hierarchy (GB300, mixed, 30
// iterations): 1,199 us per iteration unfused, 1,215 us fusing level 1 (13k entries), 1,231 us levels 1-2,
// 1,283 us levels 1-3: the separate launches overlap one another (programmatic dependent launch), a
// cluster launch waits for its predecessor to drain and for 16 free SMs.
long g_fused_jacobi_entries = 0;
// segmented batches: the cluster-fused multicolour-SOR step on concatenated levels, one cluster per group
// of whole systems; off by default.  Measured on the 96-system workload (GB300): 803 ms per batch solve
// with it against 714 ms with one launch per colour (a group's sweeps run on one cluster's 16 SMs).
int g_fused_groups = 0;
// per-level layout autotuning at upload (lina_gpu_set_autotune) for hierarchies created afterwards;
// segmented batches always tune their concatenated levels
int g_autotune = 0;
// 16: SELL-32 matrices with long rows uploaded afterwards also get 16-bit column offsets (two bases
// per slice, where every slice's columns fit), read by FP32 passes; 32: int columns only
int g_sell_bits = 16;
int g_quads = 1;  // FP32 passes read the quad layout (sellq_kernel); 0 keeps the one-entry SELL layout
int g_pdl = 1;    // programmatic dependent launch of the solve kernels (launch())
long g_mem_limit = 0;  // device bytes one handle may hold (0: no limit), lina_gpu_set_device_memory_limit
int g_coarse_device_rows = 256;      // coarsest blocks of this many rows or more are inverted on the GPU
int g_dense_method = LINA_DENSE_SIMT;  // their rank-32 updates: FP64 CUDA cores or FP64 tensor cores

void set_err(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
}

#define CK(call)                                                                   \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            set_err("%s failed: %s", #call, cudaGetErrorString(e_));               \
            return LINA_GPU_ECUDA;                                                 \
        }                                                                          \
    } while (0)

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 16384;     // partials per reduction value
constexpr int kGridCap = 152 * 12;    // grid-stride cap: 152 SMs x 12 blocks of 256
constexpr int kReduceGrid = 152 * 4;  // streaming reductions: half a wave, four strides per loop trip

// ---------------------------------------------------------------- reductions
// Programmatic dependent launch: kernels of the solve are launched with programmatic stream
// serialisation.  Each kernel first waits, before any access to global memory, until the previous grid
// has completed and its writes are visible, then lets the next kernel's blocks be scheduled: they take
// the SMs this grid's finishing blocks free and wait there, so the launch gap between the many short
// kernels of a V-cycle is hidden.  Both instructions are no-ops for a kernel launched without the
// attribute.
__device__ __forceinline__ void pdl_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum v[0..NV) over the whole grid.  Each block stores a partial; the last
// block (ticket) adds the partials in index order and calls fin(sum[]).
template <int NV, typename Fin>
__device__ void grid_reduce(double (&v)[NV], double* partials, unsigned* ticket, Fin fin) {
    __shared__ double sm[NV][32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double x = warp_sum(v[k]);
        if (lane == 0) sm[k][wid] = x;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double x = (lane < nw) ? sm[k][lane] : 0.0;
            x = warp_sum(x);
            if (lane == 0) partials[k * kMaxBlocks + blockIdx.x] = x;
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double tot[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double x = 0.0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) x += __ldcg(partials + k * kMaxBlocks + i);
        x = warp_sum(x);
        __syncthreads();
        if (lane == 0) sm[k][wid] = x;
        __syncthreads();
        double y = (lane < nw) ? sm[k][lane] : 0.0;
        tot[k] = warp_sum(y);
    }
    if (threadIdx.x == 0) {
        fin(tot);
        *ticket = 0u;
    }
}

// The block's sum of v, stored to partials[blockIdx.x] (no ticket: the SpMV+dot launches use a full
// grid, and thousands of blocks on one atomic counter cost more than a second small launch).
__device__ void block_partial(double v, double* partials) {
    __shared__ double sm[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double x = (lane < nw) ? sm[lane] : 0.0;
        x = warp_sum(x);
        if (lane == 0) partials[blockIdx.x] = x;
    }
}

// Krylov scalars kept on the device so that no host round trip sits between kernels.
constexpr int kFcgMax = 8;  // longest direction history of the truncated flexible CG
struct KScalars {
    double s, s_old, pq, t, rr, alpha, beta, r0, norm2, aux, tol;
    int iter;
    int maxit;
    double tj[kFcgMax];   // z . q_{k-j}, j = 1..m (truncated flexible CG)
    double pqh[kFcgMax];  // p_i . q_i of the kept directions, by history slot i mod m
    // Scalars derived from the reductions, formed once by the thread that finishes a reduction: FP64
    // division is slow on GB300, and each of several hundred thousand threads forming its own copy cost
    // tens of microseconds per kernel
    double cj[kFcgMax];   // FCG(m) coefficients tj / pqh
    double alpha_next;    // s / (p.q) for update_xr
};

// p.q from the block partials of an SpMV+dot launch, summed in block order by one block
__global__ void dot_finish_kernel(int nparts, const double* __restrict__ partials, KScalars* sc) {
    pdl_wait();
    __shared__ double sm[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // eight independent loads per thread per trip (the partials sit in L2), combined in a fixed order
    double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    int i = threadIdx.x;
    for (; i + 7 * (int)blockDim.x < nparts; i += 8 * blockDim.x) {
#pragma unroll
        for (int u = 0; u < 8; u++) a[u] += partials[i + u * blockDim.x];
    }
    for (; i < nparts; i += blockDim.x) a[0] += partials[i];
    double x = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    x = warp_sum(x);
    if (lane == 0) sm[wid] = x;
    __syncthreads();
    if (wid == 0) {
        double y = (lane < nw) ? sm[lane] : 0.0;
        y = warp_sum(y);
        if (lane == 0) {
            sc->pq = y;
            sc->alpha_next = sc->s / y;  // the step length of update_xr (unused by other callers)
        }
    }
}

// last node of the graph-captured iteration: continue the device-side loop
// while the residual test fails and the iteration budget lasts
__global__ void loop_cond_kernel(cudaGraphConditionalHandle handle, const KScalars* sc) {
    pdl_wait();
    const double rel = sqrt(sc->rr) / sc->r0;
    const bool more = isfinite(rel) && rel > sc->tol && sc->iter < sc->maxit;
    cudaGraphSetConditional(handle, more ? 1u : 0u);
}

// ---------------------------------------------------------------- CSR kernels
enum { M_SPMV = 0, M_RESID = 1, M_JACOBI = 2, M_SOR = 3, M_ADD = 4, M_DOT = 5 };

// SELL-32 layout: rows are cut into slices of 32 consecutive rows (of the
// natural order, or of a colour class); slice s holds its rows' entries
// column-major, entry k of the row in lane l at sptr[s] + 32 k + l, padded to
// the longest row of the slice with (own row, 0.0).  One thread per row: the
// warp's loads of values and column indices are 128-byte coalesced and every
// load of a row is independent of the others, so many are in flight.  Entries
// of a row are summed in stored (column) order.
//  M_SPMV : y = A x
//  M_RESID: y = b - A x
//  M_JACOBI: y = x + w dinv (b - A x)              (y != x)
//  M_SOR  : x = x + w dinv (b - A x) for the rows of one colour (in place)
//  M_ADD  : y = z + A x                             (z may alias y)
//  M_DOT  : y = A x, and sum_i x_i y_i -> sc->pq
// Column indices are stored either as int (TI = int) or as 16-bit offsets (TI = unsigned short):
// each slice has two bases, and an entry holds its column's offset from the first (bit 15 clear)
// or from the second (bit 15 set), 15 bits each.  The columns of a slice of 32 neighbouring rows
// fall in at most two such windows of 32,768 in the levels of P1 hierarchies (the second window
// holds the other displacement component of elasticity's component-blocked ordering), so a
// stored entry moves 6 bytes instead of 8 in FP32.  Indices are kept in registers as loaded and
// decoded only where x is gathered, so that decoding does not wait for a load issued ahead of its
// use.
__device__ __forceinline__ int sell_col(int c, int2) { return c; }
__device__ __forceinline__ int sell_col(unsigned short d, int2 base) {
    return ((d & 0x8000u) ? base.y : base.x) + (int)(d & 0x7fffu);
}

// rowseg / act (segmented batches, else null): the system of every row and whether it is still iterating;
// the rows of systems that have stopped are skipped (their values are not used any more)
template <typename TV, typename TX, int MODE, bool LONG, typename TI>
__global__ void __launch_bounds__(kThreads) sell_kernel(int npos, int nrows, const int* __restrict__ rowmap,
                                                        const int* __restrict__ sptr, const int2* __restrict__ sbase,
                                                        const TI* __restrict__ col, const TV* __restrict__ val,
                                                        const TX* x, TX* y, const TX* __restrict__ b,
                                                        const TX* __restrict__ dinv, TX w, const TX* z,
                                                        double* partials, unsigned* ticket, KScalars* sc,
                                                        const int* __restrict__ rowseg, const int* __restrict__ act) {
    pdl_wait();
    double dot = 0.0;
    // grid-stride over slice positions (npos is a multiple of 32, so warps stay whole); positions
    // past the last row (natural order) or marked -1 (colour order) are padding
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npos; t += gridDim.x * blockDim.x) {
        const int i = rowmap ? rowmap[t] : t;
        if (i < 0 || i >= nrows) continue;
        if (rowseg && !act[rowseg[i]]) continue;
        const int sl = t >> 5, lane = t & 31;
        const int p0 = sptr[sl];
        const int len = (sptr[sl + 1] - p0) >> 5;
        int2 cb = make_int2(0, 0);
        if constexpr (sizeof(TI) == 2) cb = __ldg(sbase + sl);
        const TI* cp = col + p0 + lane;
        const TV* vp = val + p0 + lane;
        TX sum = TX(0);
        int k = 0;
        // Batches of eight entries: eight index loads, eight value loads, eight gathers of x, then
        // the products in stored order, so every thread keeps several loads in flight.  LONG rows
        // (dense coarse operators) are software-pipelined: the indices and values of the next
        // batch are loaded before the gathers of the current one.  Short rows run predicated
        // batches instead (fewer registers, so more threads per SM).  The matrix streams through
        // once (evict-first loads); x is read through the read-only path (no thread reads an
        // entry of y written by another thread of the same launch, also in the in-place SOR
        // mode, where rows of one colour do not couple).
        if constexpr (LONG) {
            if (len >= 8) {
                TI c[8];
                TV v[8];
#pragma unroll
                for (int u = 0; u < 8; u++) c[u] = __ldcs(cp + 32 * u);
#pragma unroll
                for (int u = 0; u < 8; u++) v[u] = __ldcs(vp + 32 * u);
                for (k = 8;; k += 8) {
                    TX xv[8];
#pragma unroll
                    for (int u = 0; u < 8; u++) xv[u] = __ldg(x + sell_col(c[u], cb));
                    const bool more = (k + 8 <= len);
                    TI cn[8];
                    TV vn[8];
                    if (more) {
#pragma unroll
                        for (int u = 0; u < 8; u++) cn[u] = __ldcs(cp + 32 * (k + u));
#pragma unroll
                        for (int u = 0; u < 8; u++) vn[u] = __ldcs(vp + 32 * (k + u));
                    }
#pragma unroll
                    for (int u = 0; u < 8; u++) sum += TX(v[u]) * xv[u];
                    if (!more) break;
#pragma unroll
                    for (int u = 0; u < 8; u++) c[u] = cn[u], v[u] = vn[u];
                }
            }
        } else {
            for (; k + 8 <= len; k += 8) {
                TI c[8];
                TV v[8];
                TX xv[8];
#pragma unroll
                for (int u = 0; u < 8; u++) c[u] = __ldcs(cp + 32 * (k + u));
#pragma unroll
                for (int u = 0; u < 8; u++) v[u] = __ldcs(vp + 32 * (k + u));
#pragma unroll
                for (int u = 0; u < 8; u++) xv[u] = __ldg(x + sell_col(c[u], cb));
#pragma unroll
                for (int u = 0; u < 8; u++) sum += TX(v[u]) * xv[u];
            }
        }
        if (k + 4 <= len) {
            TI c[4];
            TV v[4];
            TX xv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) c[u] = __ldcs(cp + 32 * (k + u));
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = __ldcs(vp + 32 * (k + u));
#pragma unroll
            for (int u = 0; u < 4; u++) xv[u] = __ldg(x + sell_col(c[u], cb));
#pragma unroll
            for (int u = 0; u < 4; u++) sum += TX(v[u]) * xv[u];
            k += 4;
        }
        for (; k < len; k++) sum += TX(__ldcs(vp + 32 * k)) * __ldg(x + sell_col(__ldcs(cp + 32 * k), cb));
        if constexpr (MODE == M_SPMV) {
            y[i] = sum;
        } else if constexpr (MODE == M_RESID) {
            y[i] = b[i] - sum;
        } else if constexpr (MODE == M_JACOBI || MODE == M_SOR) {
            y[i] = x[i] + w * dinv[i] * (b[i] - sum);
        } else if constexpr (MODE == M_ADD) {
            y[i] = z[i] + sum;
        } else if constexpr (MODE == M_DOT) {
            y[i] = sum;
            dot += double(x[i]) * double(sum);
        }
    }
    if constexpr (MODE == M_DOT) block_partial(dot, partials);
}

// SELL-32 in quads, for the FP32 passes over natural-order matrices: slice s holds its 32 rows' entries
// in groups of four consecutive entries of a row, group g of the row in lane l at sptr[s] / 4 + 32 g + l
// (rows padded to a multiple of four with the row's own first column and value 0), values as float4 and
// the four 16-bit column offsets (bases per slice, as in sell_kernel) as one uint2.  A lane moves 24 bytes
// of matrix data per load pair where the one-entry layout moves 6, so the same registers keep four times
// as many bytes in flight: measured on the 2.1M-dof elasticity hierarchy (GB300), the FP32 sweeps of
// its long-row levels 7 and 8 went from 64-69 us to 52-60 us, level 6 from 27 to 20 us and the finest
// level (14 entries per row, padded to 16) from 44 to 37 us.  Batches of two groups (eight entries) are
// software-pipelined; at most 51 registers (five blocks of 256 per SM).  Entries are summed in stored
// order, so the results equal sell_kernel's bit for bit.
__device__ __forceinline__ int quad_col(unsigned d, int2 base) {
    return ((d & 0x8000u) ? base.y : base.x) + (int)(d & 0x7fffu);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads, 5) sellq_kernel(int n, const int* __restrict__ sptr,
                                                            const int2* __restrict__ sbase,
                                                            const uint2* __restrict__ col4,
                                                            const float4* __restrict__ val4, const float* x,
                                                            float* y, const float* __restrict__ b,
                                                            const float* __restrict__ dinv, float w,
                                                            const float* z, const int* __restrict__ rowseg,
                                                            const int* __restrict__ act) {
    pdl_wait();
    const int npos = ((n + 31) >> 5) << 5;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npos; t += gridDim.x * blockDim.x) {
        const int i = t;
        if (i >= n) continue;
        if (rowseg && !act[rowseg[i]]) continue;  // a stopped system of a segmented batch
        const int sl = t >> 5, lane = t & 31;
        const int g0 = sptr[sl] >> 2;
        const int ng = (sptr[sl + 1] - sptr[sl]) >> 7;  // groups of four per row
        const int2 cb = __ldg(sbase + sl);
        const uint2* cp = col4 + g0 + lane;
        const float4* vp = val4 + g0 + lane;
        float sum = 0.f;
        int k = 0;
        if (ng >= 2) {
            uint2 c[2];
            float4 v[2];
#pragma unroll
            for (int u = 0; u < 2; u++) c[u] = __ldcs(cp + 32 * u);
#pragma unroll
            for (int u = 0; u < 2; u++) v[u] = __ldcs(vp + 32 * u);
            for (k = 2;; k += 2) {
                float xv[8];
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    xv[4 * u + 0] = __ldg(x + quad_col(c[u].x & 0xffffu, cb));
                    xv[4 * u + 1] = __ldg(x + quad_col(c[u].x >> 16, cb));
                    xv[4 * u + 2] = __ldg(x + quad_col(c[u].y & 0xffffu, cb));
                    xv[4 * u + 3] = __ldg(x + quad_col(c[u].y >> 16, cb));
                }
                const bool more = (k + 2 <= ng);
                uint2 cn[2];
                float4 vn[2];
                if (more) {
#pragma unroll
                    for (int u = 0; u < 2; u++) cn[u] = __ldcs(cp + 32 * (k + u));
#pragma unroll
                    for (int u = 0; u < 2; u++) vn[u] = __ldcs(vp + 32 * (k + u));
                }
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    sum += v[u].x * xv[4 * u];
                    sum += v[u].y * xv[4 * u + 1];
                    sum += v[u].z * xv[4 * u + 2];
                    sum += v[u].w * xv[4 * u + 3];
                }
                if (!more) break;
#pragma unroll
                for (int u = 0; u < 2; u++) c[u] = cn[u], v[u] = vn[u];
            }
        }
        for (; k < ng; k++) {
            const uint2 c = __ldcs(cp + 32 * k);
            const float4 v = __ldcs(vp + 32 * k);
            sum += v.x * __ldg(x + quad_col(c.x & 0xffffu, cb));
            sum += v.y * __ldg(x + quad_col(c.x >> 16, cb));
            sum += v.z * __ldg(x + quad_col(c.y & 0xffffu, cb));
            sum += v.w * __ldg(x + quad_col(c.y >> 16, cb));
        }
        if constexpr (MODE == M_SPMV) {
            y[i] = sum;
        } else if constexpr (MODE == M_RESID) {
            y[i] = b[i] - sum;
        } else if constexpr (MODE == M_JACOBI) {
            y[i] = x[i] + w * dinv[i] * (b[i] - sum);
        } else if constexpr (MODE == M_ADD) {
            y[i] = z[i] + sum;
        }
    }
}

// CSR with a group of S lanes per row, for levels whose rows are long (dense
// coarse operators) or too few to fill the GPU one thread per row.  Lanes of a
// group read consecutive entries of their row (coalesced); `rows` lists the
// rows of one colour class, or is null for all rows in order.
template <typename TV, typename TX, int S, int MODE>
__global__ void __launch_bounds__(kThreads) csrv_kernel(int nrows, const int* __restrict__ rows,
                                                        const int* __restrict__ ptr, const int* __restrict__ col,
                                                        const TV* __restrict__ val, const TX* x, TX* y,
                                                        const TX* __restrict__ b, const TX* __restrict__ dinv, TX w,
                                                        const TX* z, double* partials, unsigned* ticket,
                                                        KScalars* sc) {
    pdl_wait();
    const int lane = threadIdx.x & 31;
    const int sub = lane & (S - 1);
    const long warp_global = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
    double dot = 0.0;
    for (long gb = warp_global * (32 / S); gb < nrows; gb += nwarps * (32 / S)) {
        const long g = gb + lane / S;
        const bool valid = g < nrows;
        int i = 0, s0 = 0, e0 = 0;
        if (valid) {
            i = rows ? rows[g] : (int)g;
            s0 = ptr[i];
            e0 = ptr[i + 1];
        }
        TX sum = TX(0);
        int k = s0 + sub;
        // four strides of the group at a time: independent loads in flight, products summed in order
        for (; k + 3 * S < e0; k += 4 * S) {
            const int c0 = __ldcs(col + k), c1 = __ldcs(col + k + S), c2 = __ldcs(col + k + 2 * S),
                      c3 = __ldcs(col + k + 3 * S);
            const TV v0 = __ldcs(val + k), v1 = __ldcs(val + k + S), v2 = __ldcs(val + k + 2 * S),
                     v3 = __ldcs(val + k + 3 * S);
            const TX x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
            sum += TX(v0) * x0;
            sum += TX(v1) * x1;
            sum += TX(v2) * x2;
            sum += TX(v3) * x3;
        }
        for (; k < e0; k += S) sum += TX(__ldcs(val + k)) * __ldg(x + __ldcs(col + k));
#pragma unroll
        for (int o = S / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, S);
        if (valid && sub == 0) {
            if constexpr (MODE == M_SPMV) {
                y[i] = sum;
            } else if constexpr (MODE == M_RESID) {
                y[i] = b[i] - sum;
            } else if constexpr (MODE == M_JACOBI || MODE == M_SOR) {
                y[i] = x[i] + w * dinv[i] * (b[i] - sum);
            } else if constexpr (MODE == M_ADD) {
                y[i] = z[i] + sum;
            } else if constexpr (MODE == M_DOT) {
                y[i] = sum;
                dot += double(x[i]) * double(sum);
            }
        }
    }
    if constexpr (MODE == M_DOT) block_partial(dot, partials);
}

// first pre-smoothing sweep from the zero guess: x = w dinv b (no SpMV); rows
// solved exactly by the isolated-row fix keep b / a (AMG_fix_isolated,
// LinA/Multigrid.c:1301-1319).  TB may be wider than TX (FP64 residual entering
// the FP32 V-cycle); the converted right-hand side is stored in bout if given.
template <typename TB, typename TX>
__global__ void jacobi_first_kernel(int n, const TB* __restrict__ b, const double* __restrict__ sign,
                                    const TX* __restrict__ dinv, const double* __restrict__ isoinv, TX w,
                                    TX* __restrict__ x, TX* __restrict__ bout) {
    pdl_wait();
    const long S = (long)gridDim.x * blockDim.x;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    auto one = [&](long k, double bd, TX di, double iso) {
        if (sign) bd *= sign[k];
        const TX bi = TX(bd);
        if (bout) bout[k] = bi;
        // isolated rows have a nonzero inverse, every other row +0.0: tested by its bits (an FP64
        // comparison per row would take GB300's slow FP64 pipe)
        x[k] = (__double_as_longlong(iso) != 0) ? TX(bd * iso) : w * di * bi;
    };
    for (; i + 3 * S < n; i += 4 * S) {
        double bb[4], iso[4];
        TX di[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            bb[u] = double(b[i + u * S]);
            di[u] = dinv[i + u * S];
            iso[u] = isoinv ? isoinv[i + u * S] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) one(i + u * S, bb[u], di[u], iso[u]);
    }
    for (; i < n; i += S) one(i, double(b[i]), dinv[i], isoinv ? isoinv[i] : 0.0);
}

// x = isolated-row fix (zero elsewhere), optional conversion of b
template <typename TB, typename TX>
__global__ void init_x_kernel(int n, const TB* __restrict__ b, const double* __restrict__ sign,
                              const double* __restrict__ isoinv, TX* __restrict__ x, TX* __restrict__ bout) {
    pdl_wait();
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double bd = double(b[i]);
        if (sign) bd *= sign[i];
        if (bout) bout[i] = TX(bd);
        x[i] = (isoinv && isoinv[i] != 0.0) ? TX(bd * isoinv[i]) : TX(0);
    }
}

// coarsest level: gather the block right-hand side, solve the single-nonzero rows
template <typename TX>
__global__ void coarse_gather_kernel(int n, const TX* __restrict__ b, const int* __restrict__ inblock,
                                     const int* __restrict__ blockpos, const double* __restrict__ dginv,
                                     double* __restrict__ bblk, TX* __restrict__ x) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (inblock[i])
            bblk[blockpos[i]] = double(b[i]);
        else
            x[i] = TX(double(b[i]) * dginv[i]);
    }
}

// dense FP64 GEMV with the block inverse: one warp per block row.  A block-diagonal coarsest level
// (rblk non-null: the block of each block row, its first position boff[k] and inverse offset ioff[k])
// multiplies each row by its own block only; with one block the arithmetic is the same.
template <typename TX>
__global__ void coarse_gemv_kernel(int m, const double* __restrict__ inv, const double* __restrict__ bblk,
                                   const int* __restrict__ brows, TX* __restrict__ x, const int* __restrict__ rblk,
                                   const int* __restrict__ boff, const long* __restrict__ ioff) {
    pdl_wait();
    const int lane = threadIdx.x & 31;
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < m;
         r += ((long)gridDim.x * blockDim.x) >> 5) {
        long base = r * (long)m;
        int m0 = 0, len = m;
        if (rblk) {
            const int k = rblk[r];
            m0 = boff[k];
            len = boff[k + 1] - m0;
            base = ioff[k] + (r - m0) * (long)len;
        }
        const double* row = inv + base;
        const double* bb = bblk + m0;
        double s = 0.0;
        for (int j = lane; j < len; j += 32) s += row[j] * bb[j];
        s = warp_sum(s);
        if (lane == 0) x[brows[r]] = TX(s);
    }
}

template <typename TA, typename TB>
__global__ void convert_kernel(long n, const TA* __restrict__ a, TB* __restrict__ b) {
    pdl_wait();
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = TB(a[i]);
}

__global__ void scale_kernel(long n, double* __restrict__ v, const double* __restrict__ f, int invert) {
    pdl_wait();
    __shared__ double sh;
    if (threadIdx.x == 0) sh = invert ? 1.0 / (*f) : (*f);
    __syncthreads();
    const double s = sh;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) v[i] *= s;
}

// AMG_solve helpers: b = signs * F, the isolated-row fix x_i = b_i / a_i, x += z
__global__ void mul_kernel(int n, double* __restrict__ b, const double* __restrict__ f) {
    pdl_wait();
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] *= f[i];
}

__global__ void fix_isolated_kernel(int n, const double* __restrict__ b, const double* __restrict__ isoinv,
                                    double* __restrict__ x) {
    pdl_wait();
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        if (isoinv[i] != 0.0) x[i] = b[i] * isoinv[i];
}

// new finest-level values on the setup's pattern: scatter into the level's layout(s) and
// refresh the Jacobi diagonal and the isolated-row inverses
__global__ void update_values_kernel(long nnz, const double* __restrict__ val, const int* __restrict__ posA,
                                     const int* __restrict__ posAcol, double* __restrict__ a64,
                                     float* __restrict__ a32, double* __restrict__ c64, float* __restrict__ c32,
                                     const int* __restrict__ posQ, float* __restrict__ q32) {
    pdl_wait();
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x) {
        const double v = val[k];
        const int p = posA[k];
        if (p >= 0) {
            a64[p] = v;
            a32[p] = float(v);
        }
        if (posQ) {
            const int q = posQ[k];
            if (q >= 0) q32[q] = float(v);
        }
        if (posAcol) {
            const int q = posAcol[k];
            if (q >= 0) {
                c64[q] = v;
                c32[q] = float(v);
            }
        }
    }
}

__global__ void update_diag_kernel(int n, const double* __restrict__ val, const int* __restrict__ ptr,
                                   const int* __restrict__ diagpos, const unsigned char* __restrict__ isolated,
                                   double* __restrict__ dinv64, float* __restrict__ dinv32,
                                   double* __restrict__ isoinv) {
    pdl_wait();
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int dp = diagpos[i];
        const double d = dp >= 0 ? val[dp] : 0.0;
        const double inv = d != 0.0 ? 1.0 / d : 0.0;
        dinv64[i] = inv;
        dinv32[i] = float(inv);
        double iso = 0.0;
        if (isolated[i])
            for (int q = ptr[i]; q < ptr[i + 1]; q++)
                if (val[q] != 0.0) {
                    iso = 1.0 / val[q];
                    break;
                }
        isoinv[i] = iso;
    }
}

template <typename TZ>
__global__ void add_kernel(int n, double* __restrict__ x, const TZ* __restrict__ z) {
    pdl_wait();
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        x[i] += double(z[i]);
}

// ------------------------------------------------------------ Krylov kernels
// The streaming Krylov kernels below take four grid strides per loop trip: the loads of the four
// elements are independent, so each thread keeps several in flight; partial sums are added in a
// fixed order (deterministic).

// s_old = s; s = r.z; t = z.q (flexible CG)
template <typename TZ>
__global__ void __launch_bounds__(kThreads) dot_rz_kernel(int n, const double* __restrict__ r,
                                                          const TZ* __restrict__ z, const double* __restrict__ q,
                                                          int flexible, double* partials, unsigned* ticket,
                                                          KScalars* sc) {
    pdl_wait();
    double v[2] = {0.0, 0.0};
    const long S = (long)gridDim.x * blockDim.x;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * S < n; i += 4 * S) {
        double zz[4], rr[4];
#pragma unroll
        for (int u = 0; u < 4; u++) zz[u] = double(z[i + u * S]), rr[u] = r[i + u * S];
        if (flexible) {
            double qq[4];
#pragma unroll
            for (int u = 0; u < 4; u++) qq[u] = q[i + u * S];
#pragma unroll
            for (int u = 0; u < 4; u++) v[1] += zz[u] * qq[u];
        }
#pragma unroll
        for (int u = 0; u < 4; u++) v[0] += rr[u] * zz[u];
    }
    for (; i < n; i += S) {
        const double zi = double(z[i]);
        v[0] += r[i] * zi;
        if (flexible) v[1] += zi * q[i];
    }
    grid_reduce<2>(v, partials, ticket, [sc, flexible](double* t) {
        sc->s_old = sc->s;
        sc->s = t[0];
        sc->t = t[1];
        // beta of update_p: s/s_old (CG) or -alpha_prev t / s_old (flexible CG); 0 on the first step
        sc->beta = (sc->iter == 0) ? 0.0 : flexible ? (-sc->alpha * sc->t / sc->s_old) : (sc->s / sc->s_old);
    });
}

// p = z + beta p;  beta = s/s_old (CG) or -alpha_prev t / s_old (flexible CG); p = z on the first step
template <typename TZ>
__global__ void update_p_kernel(int n, const TZ* __restrict__ z, double* __restrict__ p, int flexible,
                                KScalars* sc) {
    pdl_wait();
    const bool first = (sc->iter == 0);
    const double beta = sc->beta;  // formed by dot_rz_kernel's last block
    (void)flexible;
    const long S = (long)gridDim.x * blockDim.x;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (first) {
        for (; i < n; i += S) p[i] = double(z[i]);
        return;
    }
    for (; i + 3 * S < n; i += 4 * S) {
        double zz[4], pp[4];
#pragma unroll
        for (int u = 0; u < 4; u++) zz[u] = double(z[i + u * S]), pp[u] = p[i + u * S];
#pragma unroll
        for (int u = 0; u < 4; u++) p[i + u * S] = zz[u] + beta * pp[u];
    }
    for (; i < n; i += S) p[i] = double(z[i]) + beta * p[i];
}

// Truncated flexible CG (Notay's FCG(m)): the new direction is made A-orthogonal to the last m
// directions, p_k = z - sum_{j=1..min(k,m)} (z.q_{k-j} / p_{k-j}.q_{k-j}) p_{k-j}.  With a preconditioner
// that varies slightly between applications (the FP32 V-cycle's rounding) the longer orthogonalisation
// keeps the convergence of CG with an exact preconditioner; m = 1 is the flexible CG above.  The
// kept directions p_i and q_i = A p_i live in rings of m slots (slot i mod m), written by
// update_xr_kernel; the slots are found from the device's iteration counter, so the captured graph
// needs no pointer changes.

// s_old = s; s = r.z; tj[j-1] = z.q_{k-j}, j = 1..min(k, M)
template <typename TZ, int M>
__global__ void __launch_bounds__(kThreads, 4) fcg_dot_kernel(int n, const double* __restrict__ r,
                                                           const TZ* __restrict__ z, const double* __restrict__ qh,
                                                           double* partials, unsigned* ticket, KScalars* sc) {
    pdl_wait();
    const int k = sc->iter;
    const int nprev = k < M ? k : M;
    const double* qs[M];
#pragma unroll
    for (int j = 1; j <= M; j++) qs[j - 1] = qh + (size_t)((k - j + M * kFcgMax) % M) * n;
    double v[M + 1];
#pragma unroll
    for (int j = 0; j <= M; j++) v[j] = 0.0;
    // U grid strides per loop trip, all loads of a trip issued before the products (independent loads
    // in flight); the sums are taken in a fixed order
    constexpr int U = (M <= 3) ? 4 : 2;
    const long S = (long)gridDim.x * blockDim.x;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (U - 1) * S < n; i += U * S) {
        double zz[U], rr[U], qq[M][U];
#pragma unroll
        for (int u = 0; u < U; u++) zz[u] = double(z[i + u * S]), rr[u] = r[i + u * S];
#pragma unroll
        for (int j = 1; j <= M; j++)
#pragma unroll
            for (int u = 0; u < U; u++) qq[j - 1][u] = (j <= nprev) ? qs[j - 1][i + u * S] : 0.0;
#pragma unroll
        for (int u = 0; u < U; u++) {
            v[0] += rr[u] * zz[u];
#pragma unroll
            for (int j = 1; j <= M; j++) v[j] += zz[u] * qq[j - 1][u];
        }
    }
    for (; i < n; i += S) {
        const double zi = double(z[i]);
        v[0] += r[i] * zi;
#pragma unroll
        for (int j = 1; j <= M; j++)
            if (j <= nprev) v[j] += zi * qs[j - 1][i];
    }
    grid_reduce<M + 1>(v, partials, ticket, [sc, k, nprev](double* t) {
        sc->s_old = sc->s;
        sc->s = t[0];
#pragma unroll
        for (int j = 1; j <= M; j++) {
            sc->tj[j - 1] = t[j];
            sc->cj[j - 1] = (j <= nprev) ? t[j] / sc->pqh[(k - j + M * kFcgMax) % M] : 0.0;
        }
    });
}

// p_k = z - sum_j (tj[j-1] / pqh[(k-j) mod M]) p_{k-j}
template <typename TZ, int M>
__global__ void __launch_bounds__(kThreads, 4) fcg_update_p_kernel(int n, const TZ* __restrict__ z, const double* __restrict__ ph,
                                    double* __restrict__ p, const KScalars* sc) {
    pdl_wait();
    const int k = sc->iter;
    const int nprev = k < M ? k : M;
    double c[M];
    const double* ps[M];
#pragma unroll
    for (int j = 1; j <= M; j++) {
        const int slot = (k - j + M * kFcgMax) % M;
        c[j - 1] = sc->cj[j - 1];  // formed by fcg_dot_kernel's last block
        ps[j - 1] = ph + (size_t)slot * n;
    }
    constexpr int U = (M <= 3) ? 4 : 2;
    const long S = (long)gridDim.x * blockDim.x;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (U - 1) * S < n; i += U * S) {
        double pp[U], hh[M][U];
#pragma unroll
        for (int u = 0; u < U; u++) pp[u] = double(z[i + u * S]);
#pragma unroll
        for (int j = 1; j <= M; j++)
#pragma unroll
            for (int u = 0; u < U; u++) hh[j - 1][u] = (j <= nprev) ? ps[j - 1][i + u * S] : 0.0;
#pragma unroll
        for (int u = 0; u < U; u++) {
#pragma unroll
            for (int j = 1; j <= M; j++) pp[u] -= c[j - 1] * hh[j - 1][u];
            p[i + u * S] = pp[u];
        }
    }
    for (; i < n; i += S) {
        double pi = double(z[i]);
#pragma unroll
        for (int j = 1; j <= M; j++)
            if (j <= nprev) pi -= c[j - 1] * ps[j - 1][i];
        p[i] = pi;
    }
}

// alpha = s / (p.q); x += alpha p; r -= alpha q; rr = r.r.  With a direction history (hm > 0) p and
// q are also stored in slot iter mod hm of the rings ph, qh, and p.q in sc->pqh.
__global__ void __launch_bounds__(kThreads, 4) update_xr_kernel(int n, double* __restrict__ x, double* __restrict__ r,
                                                             const double* __restrict__ p,
                                                             const double* __restrict__ q, double* partials,
                                                             unsigned* ticket, KScalars* sc, int hm,
                                                             double* __restrict__ ph, double* __restrict__ qh) {
    pdl_wait();
    const double alpha = sc->alpha_next;  // s / (p.q), formed by dot_finish_kernel
    double* hp = nullptr;
    double* hq = nullptr;
    if (hm > 0) {
        const size_t slot = (size_t)(sc->iter % hm);
        hp = ph + slot * n;
        hq = qh + slot * n;
    }
    double v[1] = {0.0};
    const long S = (long)gridDim.x * blockDim.x;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * S < n; i += 4 * S) {
        double xx[4], pp[4], rr[4], qq[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            xx[u] = x[i + u * S];
            pp[u] = p[i + u * S];
            rr[u] = r[i + u * S];
            qq[u] = q[i + u * S];
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            x[i + u * S] = xx[u] + alpha * pp[u];
            const double ri = rr[u] - alpha * qq[u];
            r[i + u * S] = ri;
            v[0] += ri * ri;
        }
        if (hp) {
#pragma unroll
            for (int u = 0; u < 4; u++) {
                hp[i + u * S] = pp[u];
                hq[i + u * S] = qq[u];
            }
        }
    }
    for (; i < n; i += S) {
        const double pi = p[i], qi = q[i];
        x[i] += alpha * pi;
        const double ri = r[i] - alpha * qi;
        r[i] = ri;
        v[0] += ri * ri;
        if (hp) {
            hp[i] = pi;
            hq[i] = qi;
        }
    }
    grid_reduce<1>(v, partials, ticket, [sc, alpha, hm](double* t) {
        sc->rr = t[0];
        sc->alpha = alpha;
        if (hm > 0) sc->pqh[sc->iter % hm] = sc->pq;
        sc->iter += 1;
    });
}

template <typename T>
__global__ void __launch_bounds__(kThreads) norm2_kernel(int n, const T* __restrict__ v, double* partials,
                                                         unsigned* ticket, KScalars* sc) {
    pdl_wait();
    double a[1] = {0.0};
    const long S = (long)gridDim.x * blockDim.x;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * S < n; i += 4 * S) {
        double w[4];
#pragma unroll
        for (int u = 0; u < 4; u++) w[u] = double(v[i + u * S]);
#pragma unroll
        for (int u = 0; u < 4; u++) a[0] += w[u] * w[u];
    }
    for (; i < n; i += S) {
        const double x = double(v[i]);
        a[0] += x * x;
    }
    grid_reduce<1>(a, partials, ticket, [sc](double* t) { sc->norm2 = t[0]; });
}

}  // namespace

// ======================================================================= host
namespace {

// a matrix on the device in SELL-32 layout (see sell_kernel)
// ------------------------------------------------------------ cluster-fused V-cycle steps
// On small levels a multicolour-SOR sweep is a chain of tiny launches (one per colour: 10-25 on the
// coarse levels of elasticity hierarchies), each bound by launch and memory latency.  A level step
// instead runs as one launch of a thread-block cluster:
//   pre : x = 0 | sweep colour 0 | ... | colour c-1 (nu times) | r = b - A x | b_coarse = R r
//   post: x += P e | sweep colour 0 | ... (nu times)
// with a cluster barrier where the separate launches had a kernel boundary.  Every block keeps a
// full copy of the level's x in its shared memory for the whole step: a row reads its neighbours
// from its own SM, and a new entry is stored into every block's copy (the lanes of the row's group
// share those stores) before the colour's barrier.  x is read from and written back to global
// memory once per step.  Every row is computed exactly as csrv_kernel computes it (the same lane
// groups, the same order of products and of the shuffle reduction), so the results are
// bit-identical to the per-colour launches.
namespace cg = cooperative_groups;

constexpr int kFuseThreads = 512;
constexpr int kFusedSmemMax = 192 * 1024;  // a block's copy of x: 49,152 FP32 or 24,576 FP64 rows

struct FusedStep {
    int n, nc, ncolours, nu;
    int sS, aS, rS, pS;  // lanes per row: colour-grouped A, natural A, R, P
    const int *sptr, *scol, *srows, *sgroup;
    const int4* shead;  // (row, first entry, end of entries) per position of the colour order
    const int *aptr, *acol;
    const int *rptr, *rcol;
    const int *pptr, *pcol;
    const void *sval, *aval, *rval, *pval, *dinv, *b, *e;
    void *x, *r, *cb;
    double w;
};

// A cluster's share of a level made of independent systems (a segmented batch): the rows [r0, r1) of
// whole systems, their coarse rows [c0, c1), and at granges + c the positions of its rows of colour c in
// the colour order.  Its rows couple only to its own rows, so each cluster sweeps on its own.
struct FusedGroup {
    int r0, r1, c0, c1;
    const int2* granges;
};

// a block's copy of x, holding the rows [off, off + rows) of the level
template <typename TX>
struct LocalRead {
    const TX* p;
    int off;
    __device__ __forceinline__ TX get(int j) const { return p[j - off]; }
};
template <typename TX>
struct GlobalRead {
    const TX* p;
    __device__ __forceinline__ TX get(int j) const { return __ldcg(p + j); }
};

// entry i of every block's copy of x := v, the group's S lanes sharing the stores
template <typename TX>
__device__ __forceinline__ void broadcast_x(TX* xs, int i, TX v, int sub, int S, int off = 0) {
    const cg::cluster_group cl = cg::this_cluster();
    const int K = (int)cl.num_blocks();
    if (K == 1) {
        if (sub == 0) xs[i - off] = v;
        return;
    }
    for (int r = sub; r < K; r += S) cl.map_shared_rank(xs, (unsigned)r)[i - off] = v;
}

// the barrier between phases of a fused step: a block barrier where the cluster is one block
__device__ __forceinline__ void fused_sync(const cg::cluster_group& cl) {
    if (cl.num_blocks() == 1)
        __syncthreads();
    else
        cl.sync();
}

// sum_k val_k v_col_k over one row by a group of S lanes (the order of csrv_kernel); the butterfly
// leaves the sum in every lane of the group
template <typename TX, typename V>
__device__ __forceinline__ TX fused_row_sum(bool valid, int s0, int e0, int sub, int S, const int* __restrict__ col,
                                            const TX* __restrict__ val, const V& v) {
    TX sum = TX(0);
    if (valid) {
        int k = s0 + sub;
        for (; k + 3 * S < e0; k += 4 * S) {
            const int c0 = __ldg(col + k), c1 = __ldg(col + k + S), c2 = __ldg(col + k + 2 * S),
                      c3 = __ldg(col + k + 3 * S);
            const TX v0 = __ldg(val + k), v1 = __ldg(val + k + S), v2 = __ldg(val + k + 2 * S),
                     v3 = __ldg(val + k + 3 * S);
            const TX x0 = v.get(c0), x1 = v.get(c1), x2 = v.get(c2), x3 = v.get(c3);
            sum += TX(v0) * x0;
            sum += TX(v1) * x1;
            sum += TX(v2) * x2;
            sum += TX(v3) * x3;
        }
        for (; k < e0; k += S) sum += TX(__ldg(val + k)) * v.get(__ldg(col + k));
    }
    for (int o = S / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, S);
    return sum;
}

// rows [r0, r1) of the natural order in lane groups of S spread over the cluster; f(i, sum, sub)
// is called by every lane of row i's group
template <typename TX, typename V, typename F>
__device__ __forceinline__ void fused_rows(int r0, int r1, int S, const int* __restrict__ ptr,
                                           const int* __restrict__ col, const TX* __restrict__ val, const V& v,
                                           F f) {
    const int lane = threadIdx.x & 31, sub = lane & (S - 1);
    const cg::cluster_group cl = cg::this_cluster();
    const int warp = (int)(cl.thread_rank() >> 5), nwarps = (int)(cl.num_threads() >> 5);
    const int per_warp = 32 / S;
    for (int gb = r0 + warp * per_warp; gb < r1; gb += nwarps * per_warp) {
        const int g = gb + lane / S;
        const bool valid = g < r1;
        int s0 = 0, e0 = 0;
        if (valid) {
            s0 = __ldg(ptr + g);
            e0 = __ldg(ptr + g + 1);
        }
        const TX sum = fused_row_sum<TX>(valid, s0, e0, sub, S, col, val, v);
        if (valid) f(g, sum, sub);
    }
}

// The first row a lane group sweeps in a colour, fetched before the colour starts: everything
// but the entries of x, which the previous colour may have changed.
template <typename TX>
struct SweepRow {
    int i = 0, s0 = 0, e0 = 0;
    int c[4];
    TX v[4];
    TX bi = TX(0), di = TX(0);
};

// the row at position g of the colour order: its head (row and entry range) is loaded one step
// before the rest, so that no load of a step depends on another load of the same step
template <typename TX>
__device__ __forceinline__ int4 load_head(const FusedStep& st, int g, bool valid) {
    return valid ? __ldg(st.shead + g) : make_int4(0, 0, 0, 0);
}

template <typename TX>
__device__ __forceinline__ void build_sweep_row(SweepRow<TX>& p, int4 h, bool valid, int sub, int S,
                                                const FusedStep& st, const TX* __restrict__ sval,
                                                const TX* __restrict__ b, const TX* __restrict__ dinv) {
    p.i = h.x;
    p.s0 = h.y;
    p.e0 = h.z;
    if (valid) {
        p.bi = __ldg(b + p.i);
        p.di = __ldg(dinv + p.i);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int k = p.s0 + sub + j * S;
        const bool in = valid && k < p.e0;
        p.c[j] = in ? __ldg(st.scol + k) : -1;
        p.v[j] = in ? __ldg(sval + k) : TX(0);
    }
}

template <typename TX>
__device__ __forceinline__ void fetch_sweep_row(SweepRow<TX>& p, bool valid, int g, int sub, int S,
                                                const FusedStep& st, const TX* __restrict__ sval,
                                                const TX* __restrict__ b, const TX* __restrict__ dinv) {
    build_sweep_row<TX>(p, load_head<TX>(st, g, valid), valid, sub, S, st, sval, b, dinv);
}

// the SOR update of a fetched row (the order of products of fused_row_sum: the first four strides
// from the fetched entries, the rest as csrv_kernel walks them), stored into every copy of x
template <typename TX>
__device__ __forceinline__ void sweep_fetched_row(const SweepRow<TX>& p, bool valid, int sub, int S, TX w,
                                                  const FusedStep& st, const TX* __restrict__ sval, TX* xs,
                                                  int off = 0) {
    TX sum = TX(0);
    if (valid) {
        TX xv[4];
#pragma unroll
        for (int j = 0; j < 4; j++) xv[j] = p.c[j] >= 0 ? xs[p.c[j] - off] : TX(0);
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (p.c[j] >= 0) sum += TX(p.v[j]) * xv[j];
        int k = p.s0 + sub + 4 * S;
        for (; k + 3 * S < p.e0; k += 4 * S) {
            const int c0 = __ldg(st.scol + k), c1 = __ldg(st.scol + k + S), c2 = __ldg(st.scol + k + 2 * S),
                      c3 = __ldg(st.scol + k + 3 * S);
            const TX v0 = __ldg(sval + k), v1 = __ldg(sval + k + S), v2 = __ldg(sval + k + 2 * S),
                     v3 = __ldg(sval + k + 3 * S);
            const TX x0 = xs[c0 - off], x1 = xs[c1 - off], x2 = xs[c2 - off], x3 = xs[c3 - off];
            sum += TX(v0) * x0;
            sum += TX(v1) * x1;
            sum += TX(v2) * x2;
            sum += TX(v3) * x3;
        }
        for (; k < p.e0; k += S) sum += TX(__ldg(sval + k)) * xs[__ldg(st.scol + k) - off];
    }
    for (int o = S / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, S);
    if (valid) broadcast_x(xs, p.i, xs[p.i - off] + w * p.di * (p.bi - sum), sub, S, off);
}

__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// nu sweeps over the colours, a cluster barrier after each colour.  The first row a lane group
// sweeps in a colour is loaded as a two-stage pipeline across the barriers: its head two colours
// ahead, its entries, b and 1/a_ii one colour ahead, so after a barrier only shared-memory reads of
// x are on the critical path.  Colours with more rows than the cluster has lane groups sweep the
// remaining rows directly.
// off: the first row of the level the block's copy of x holds; granges: per colour the position range
// of the cluster's rows in the colour order (null: the whole colour, st.sgroup)
template <typename TX>
__device__ __forceinline__ void fused_sweeps(const FusedStep& st, TX* xs, const TX* __restrict__ b,
                                             const TX* __restrict__ dinv, int off = 0,
                                             const int2* __restrict__ granges = nullptr) {
    const TX w = TX(st.w);
    const TX* sval = (const TX*)st.sval;
    const int S = st.sS;
    const int lane = threadIdx.x & 31, sub = lane & (S - 1);
    const cg::cluster_group cl = cg::this_cluster();
    const int warp = (int)(cl.thread_rank() >> 5), nwarps = (int)(cl.num_threads() >> 5);
    const int per_warp = 32 / S;
    const int first = warp * per_warp + lane / S;  // the group's row offset in a colour's first pass
    const int steps = st.nu * st.ncolours;
    if (steps == 0) return;
    // colour of a step and its position range
    auto range = [&](int step, int& r0, int& r1) {
        const int c = step % st.ncolours;
        if (granges) {
            const int2 g = __ldg(granges + c);
            r0 = g.x;
            r1 = g.y;
        } else {
            r0 = __ldg(st.sgroup + c);
            r1 = __ldg(st.sgroup + c + 1);
        }
    };
    int r0, r1, n0, n1, m0, m1;
    range(0, r0, r1);
    SweepRow<TX> cur, nxt;
    fetch_sweep_row<TX>(cur, r0 + first < r1, r0 + first, sub, S, st, sval, b, dinv);
    int4 h1 = make_int4(0, 0, 0, 0);
    n0 = n1 = 0;
    if (steps > 1) {
        range(1, n0, n1);
        h1 = load_head<TX>(st, n0 + first, n0 + first < n1);
    }
    for (int step = 0; step < steps; step++) {
        int4 h2 = make_int4(0, 0, 0, 0);
        m0 = m1 = 0;
        if (step + 2 < steps) {
            range(step + 2, m0, m1);
            h2 = load_head<TX>(st, m0 + first, m0 + first < m1);
        }
        if (step + 1 < steps) build_sweep_row<TX>(nxt, h1, n0 + first < n1, sub, S, st, sval, b, dinv);
        sweep_fetched_row<TX>(cur, r0 + first < r1, sub, S, w, st, sval, xs, off);
        for (int gb = r0 + warp * per_warp + nwarps * per_warp; gb < r1; gb += nwarps * per_warp) {
            const int g = gb + lane / S;
            SweepRow<TX> q;
            fetch_sweep_row<TX>(q, g < r1, g, sub, S, st, sval, b, dinv);
            sweep_fetched_row<TX>(q, g < r1, sub, S, w, st, sval, xs, off);
        }
        if (cl.num_blocks() == 1) {
            __syncthreads();
        } else {
            cluster_arrive();
            cluster_wait();
        }
        cur = nxt;
        r0 = n0;
        r1 = n1;
        h1 = h2;
        n0 = m0;
        n1 = m1;
    }
}

// nu damped-Jacobi sweeps y = x + w dinv (b - A x): each row's sum over the natural-order lane groups
// (the order of csrv_kernel), read from the block's copy cur and stored into every block's copy nxt; a
// cluster barrier after each sweep.  Returns the copy holding the result.
template <typename TX>
__device__ __forceinline__ TX* fused_jacobi_sweeps(const FusedStep& st, int nu, TX* cur, TX* nxt,
                                                   const TX* __restrict__ b, const TX* __restrict__ dinv) {
    const TX w = TX(st.w);
    const cg::cluster_group cl = cg::this_cluster();
    for (int k = 0; k < nu; k++) {
        fused_rows<TX>(0, st.n, st.aS, st.aptr, st.acol, (const TX*)st.aval, LocalRead<TX>{cur},
                       [&](int i, TX sum, int sub) {
                           broadcast_x(nxt, i, cur[i] + w * __ldg(dinv + i) * (__ldg(b + i) - sum), sub, st.aS);
                       });
        fused_sync(cl);
        TX* t = cur;
        cur = nxt;
        nxt = t;
    }
    return cur;
}

// dynamic shared memory of a block: a copy of x (n entries), two for damped Jacobi (JAC)
template <typename TX, bool PRE, bool JAC>
__global__ void __launch_bounds__(kFuseThreads, 1) fused_step_kernel(const FusedStep st,
                                                                     const FusedGroup* __restrict__ groups) {
    pdl_wait();
    extern __shared__ __align__(16) unsigned char fused_smem[];
    const cg::cluster_group cl = cg::this_cluster();
    TX* xs = reinterpret_cast<TX*>(fused_smem);
    TX* xg = (TX*)st.x;
    const TX* b = (const TX*)st.b;
    const TX* dinv = (const TX*)st.dinv;
    if constexpr (JAC) {
        // Jacobi: the first pre-sweep from the zero guess needs no product (x = w dinv b, as
        // jacobi_first_kernel), so every block forms all of it in its own copy
        TX* other = xs + st.n;
        const TX w = TX(st.w);
        for (int j = (int)threadIdx.x; j < st.n; j += blockDim.x)
            xs[j] = PRE ? (st.nu > 0 ? w * __ldg(dinv + j) * __ldg(b + j) : TX(0)) : __ldcg(xg + j);
        fused_sync(cl);  // every block runs before any remote store
        TX* res;
        if (PRE) {
            res = fused_jacobi_sweeps<TX>(st, st.nu > 0 ? st.nu - 1 : 0, xs, other, b, dinv);
            TX* r = (TX*)st.r;
            fused_rows<TX>(0, st.n, st.aS, st.aptr, st.acol, (const TX*)st.aval, LocalRead<TX>{res},
                           [&](int i, TX sum, int sub) {
                               if (sub == 0) r[i] = b[i] - sum;
                           });
            fused_sync(cl);
            TX* cb = (TX*)st.cb;
            fused_rows<TX>(0, st.nc, st.rS, st.rptr, st.rcol, (const TX*)st.rval, GlobalRead<TX>{r},
                           [&](int i, TX sum, int sub) {
                               if (sub == 0) cb[i] = sum;
                           });
        } else {
            fused_rows<TX>(0, st.n, st.pS, st.pptr, st.pcol, (const TX*)st.pval, GlobalRead<TX>{(const TX*)st.e},
                           [&](int i, TX sum, int sub) { broadcast_x(xs, i, xs[i] + sum, sub, st.pS); });
            fused_sync(cl);
            res = fused_jacobi_sweeps<TX>(st, st.nu, xs, other, b, dinv);
        }
        // the last sweep (or the start) ended with a cluster barrier: every copy of res is final
        const int chunk = (st.n + (int)cl.num_blocks() - 1) / (int)cl.num_blocks();
        const int lo = (int)cl.block_rank() * chunk, hi = min(st.n, lo + chunk);
        for (int j = lo + (int)threadIdx.x; j < hi; j += blockDim.x) xg[j] = res[j];
        fused_sync(cl);  // no block leaves while another may still store into its shared memory
        return;
    }
    // the cluster's rows: a group of whole systems (groups non-null), else the whole level
    int r0 = 0, r1 = st.n, c0 = 0, c1 = st.nc;
    const int2* granges = nullptr;
    if (groups) {
        const FusedGroup& g = groups[blockIdx.x / cl.num_blocks()];
        r0 = g.r0;
        r1 = g.r1;
        c0 = g.c0;
        c1 = g.c1;
        granges = g.granges;
    }
    const int nr = r1 - r0;
    for (int j = (int)threadIdx.x; j < nr; j += blockDim.x) xs[j] = PRE ? TX(0) : __ldcg(xg + r0 + j);
    fused_sync(cl);
    if (PRE) {
        fused_sweeps<TX>(st, xs, b, dinv, r0, granges);
        TX* r = (TX*)st.r;
        fused_rows<TX>(r0, r1, st.aS, st.aptr, st.acol, (const TX*)st.aval, LocalRead<TX>{xs, r0},
                       [&](int i, TX sum, int sub) {
                           if (sub == 0) r[i] = b[i] - sum;
                       });
        fused_sync(cl);
        TX* cb = (TX*)st.cb;
        fused_rows<TX>(c0, c1, st.rS, st.rptr, st.rcol, (const TX*)st.rval, GlobalRead<TX>{r},
                       [&](int i, TX sum, int sub) {
                           if (sub == 0) cb[i] = sum;
                       });
    } else {
        fused_rows<TX>(r0, r1, st.pS, st.pptr, st.pcol, (const TX*)st.pval, GlobalRead<TX>{(const TX*)st.e},
                       [&](int i, TX sum, int sub) { broadcast_x(xs, i, xs[i - r0] + sum, sub, st.pS, r0); });
        fused_sync(cl);
        fused_sweeps<TX>(st, xs, b, dinv, r0, granges);
    }
    // the sweeps ended with a cluster barrier: every copy is final; each block writes its share
    const int chunk = (nr + (int)cl.num_blocks() - 1) / (int)cl.num_blocks();
    const int lo = (int)cl.block_rank() * chunk, hi = min(nr, lo + chunk);
    for (int j = lo + (int)threadIdx.x; j < hi; j += blockDim.x) xg[r0 + j] = xs[j];
    fused_sync(cl);  // no block leaves while another may still store into its shared memory
}

// ------------------------------------------------------------ staged fused steps
// A fused step whose sweeps read nothing but shared memory.  At upload the level's rows are dealt to
// the K blocks of a cluster colour by colour (each block takes a contiguous share of every colour's
// rows) and each block's share is packed into two fixed-size images: ints (per colour the block's first
// local position, then its rows, their entry offsets and their columns) and values (the rows' entries,
// then omega / a_ii; gathered again on the device whenever the level's values or omega change).  A step
// copies its block's images into shared memory with asynchronous copies issued before it waits for the
// previous kernel, gathers b for its rows, and sweeps colour by colour from shared memory: the only
// traffic of a colour is the new entries of x, stored into every block's copy, and a cluster barrier (a
// block barrier where K is 1).  The pre-step's residual is summed from the images too where the natural
// matrix has the same lane groups; restriction and prolongation read R, P and the vectors from global
// memory as the unstaged step does.  Rows are summed by the lane groups and in the order of csrv_kernel,
// so results are bit-identical to the per-colour launches.
constexpr int kStagedSmemMax = 210 * 1024;

struct StagedPlan {
    const int* img;    // K int images of `ints` ints
    const void* vals;  // K value images of `nvals` values (TX)
    int ints, nvals;
    int pslots;               // b slots (the largest share's positions, a multiple of 4)
    int o_row, o_off, o_col;  // sections of an int image
    int o_dinv;               // 1/a_ii in a value image
    int xbytes;               // the copy of x, a multiple of 16 bytes
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// sum_k val_k x_col_k over entries [k0, k1) of the shared images by a group of S lanes, in the order of
// csrv_kernel; the butterfly leaves the sum in every lane of the group
template <typename TX>
__device__ __forceinline__ TX staged_row_sum(bool valid, int k0, int k1, int sub, int S, const int* scol,
                                             const TX* sv, const TX* xs) {
    TX sum = TX(0);
    if (valid) {
        // eight, then four strides at a time: the loads of a batch are in flight together (the sums
        // stay in order)
        int k = k0 + sub;
        for (; k + 7 * S < k1; k += 8 * S) {
            int c[8];
            TX v[8], x[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                c[j] = scol[k + j * S];
                v[j] = sv[k + j * S];
            }
#pragma unroll
            for (int j = 0; j < 8; j++) x[j] = xs[c[j]];
#pragma unroll
            for (int j = 0; j < 8; j++) sum += v[j] * x[j];
        }
        if (k + 3 * S < k1) {
            const int c0 = scol[k], c1 = scol[k + S], c2 = scol[k + 2 * S], c3 = scol[k + 3 * S];
            const TX v0 = sv[k], v1 = sv[k + S], v2 = sv[k + 2 * S], v3 = sv[k + 3 * S];
            const TX x0 = xs[c0], x1 = xs[c1], x2 = xs[c2], x3 = xs[c3];
            sum += v0 * x0;
            sum += v1 * x1;
            sum += v2 * x2;
            sum += v3 * x3;
            k += 4 * S;
        }
        for (; k < k1; k += S) sum += sv[k] * xs[scol[k]];
    }
    for (int o = S / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, S);
    return sum;
}

// f(q, sum, sub) for every local position q of [q0, q1), called by every lane of its group.  Consecutive
// positions share a warp: an FP64 instruction costs the SM's FP64 pipe the same with one active lane as
// with 32, so rows are packed into as few warps as possible.
template <typename TX, typename F>
__device__ __forceinline__ void staged_rows(int q0, int q1, int S, const int* soff, const int* scol, const TX* sv,
                                            const TX* xs, F f) {
    const int lane = threadIdx.x & 31, sub = lane & (S - 1);
    const int warp = (int)(threadIdx.x >> 5), nwarps = (int)(blockDim.x >> 5);
    const int per_warp = 32 / S;
    for (int qb = q0 + warp * per_warp; qb < q1; qb += nwarps * per_warp) {
        const int q = qb + lane / S;
        const bool valid = q < q1;
        const TX sum = staged_row_sum<TX>(valid, valid ? soff[q] : 0, valid ? soff[q + 1] : 0, sub, S, scol, sv, xs);
        if (valid) f(q, sum, sub);
    }
}

template <typename TX, bool PRE>
__global__ void __launch_bounds__(kFuseThreads, 1) staged_step_kernel(const FusedStep st, const StagedPlan sp) {
    extern __shared__ __align__(16) unsigned char staged_smem[];
    const cg::cluster_group cl = cg::this_cluster();
    const int K = (int)cl.num_blocks(), rank = (int)cl.block_rank();
    TX* xs = reinterpret_cast<TX*>(staged_smem);
    TX* sv = reinterpret_cast<TX*>(staged_smem + sp.xbytes);
    TX* sb = sv + sp.nvals;
    int* si = reinterpret_cast<int*>(sb + sp.pslots);
    {  // the block's images (static between value refreshes): copied while the previous kernel drains
        const char* gi = reinterpret_cast<const char*>(sp.img + (long)rank * sp.ints);
        const char* gv = reinterpret_cast<const char*>(static_cast<const TX*>(sp.vals) + (long)rank * sp.nvals);
        const int ni = sp.ints / 4, nv = sp.nvals * (int)sizeof(TX) / 16;
        for (int j = (int)threadIdx.x; j < ni; j += blockDim.x) cp_async16(reinterpret_cast<char*>(si) + 16 * j, gi + 16 * j);
        for (int j = (int)threadIdx.x; j < nv; j += blockDim.x) cp_async16(reinterpret_cast<char*>(sv) + 16 * j, gv + 16 * j);
    }
    pdl_wait();
    TX* xg = (TX*)st.x;
    const TX* b = (const TX*)st.b;
    for (int j = (int)threadIdx.x; j < st.n; j += blockDim.x) xs[j] = PRE ? TX(0) : __ldcg(xg + j);
    cp_async_wait_all();
    __syncthreads();
    const int C = st.ncolours, P = si[C];
    const int *srow = si + sp.o_row, *soff = si + sp.o_off, *scol = si + sp.o_col;
    const TX* swdi = sv + sp.o_dinv;  // omega / a_ii
    for (int q = (int)threadIdx.x; q < P; q += blockDim.x) sb[q] = __ldg(b + srow[q]);
    fused_sync(cl);  // every copy of x is set before any remote store
    if (!PRE) {
        fused_rows<TX>(0, st.n, st.pS, st.pptr, st.pcol, (const TX*)st.pval, GlobalRead<TX>{(const TX*)st.e},
                       [&](int i, TX sum, int sub) { broadcast_x(xs, i, xs[i] + sum, sub, st.pS); });
        fused_sync(cl);
    }
    const int S = st.sS;
    const int steps = st.nu * C;
    for (int step = 0; step < steps; step++) {
        const int c = step % C;
        staged_rows<TX>(si[c], si[c + 1], S, soff, scol, sv, xs, [&](int q, TX sum, int sub) {
            const int i = srow[q];
            broadcast_x(xs, i, xs[i] + swdi[q] * (sb[q] - sum), sub, S);
        });
        fused_sync(cl);
    }
    if (PRE) {
        TX* r = (TX*)st.r;
        if (st.aS == S) {  // the natural matrix sums its rows in the same lane groups: from the images
            staged_rows<TX>(0, P, S, soff, scol, sv, xs, [&](int q, TX sum, int sub) {
                if (sub == 0) r[srow[q]] = sb[q] - sum;
            });
        } else {
            fused_rows<TX>(0, st.n, st.aS, st.aptr, st.acol, (const TX*)st.aval, LocalRead<TX>{xs, 0},
                           [&](int i, TX sum, int sub) {
                               if (sub == 0) r[i] = b[i] - sum;
                           });
        }
        fused_sync(cl);
        TX* cb = (TX*)st.cb;
        fused_rows<TX>(0, st.nc, st.rS, st.rptr, st.rcol, (const TX*)st.rval, GlobalRead<TX>{r},
                       [&](int i, TX sum, int sub) {
                           if (sub == 0) cb[i] = sum;
                       });
    }
    // the sweeps ended with a barrier: every copy is final; each block writes its share
    const int chunk = (st.n + K - 1) / K;
    const int lo = rank * chunk, hi = min(st.n, lo + chunk);
    for (int j = lo + (int)threadIdx.x; j < hi; j += blockDim.x) xg[j] = xs[j];
    fused_sync(cl);  // no block leaves while another may still store into its shared memory
}

// the value images of a staged level from its colour-grouped matrix and 1/a_ii: src >= 0 an entry,
// src <= -2 omega / a_ii of row -2 - src (the product the sweep forms first: w * dinv[i] * (b[i] - sum)
// associates as (w * dinv[i]) * (...)), -1 padding
__global__ void stage_gather_kernel(long n, const int* __restrict__ src, const double* __restrict__ a64,
                                    const float* __restrict__ a32, const double* __restrict__ d64,
                                    const float* __restrict__ d32, double w, double* __restrict__ o64,
                                    float* __restrict__ o32) {
    pdl_wait();
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int s = src[i];
        double v = 0.0;
        float f = 0.f;
        if (s >= 0) {
            v = a64[s];
            f = a32[s];
        } else if (s <= -2) {
            v = w * d64[-2 - s];
            f = float(w) * d32[-2 - s];
        }
        o64[i] = v;
        o32[i] = f;
    }
}

struct DCsr {
    int n = 0, ncols = 0;
    long nnz = 0;        // stored entries of the CSR source
    long padded = 0;     // entries including slice padding
    int npos = 0;        // slice positions (multiple of 32)
    bool long_rows = false;  // mean row length >= 24: the software-pipelined SELL variant
    int* sptr = nullptr;
    int* col = nullptr;
    unsigned short* col16 = nullptr;  // 16-bit column offsets (see sell_kernel), or null
    int2* sbase = nullptr;            // the two bases of each slice for col16
    double* v64 = nullptr;
    float* v32 = nullptr;
    int* rowmap = nullptr;          // row of each position (-1 = padding), null = natural order
    // segmented batches: the system of every row and the per-system iterating flags (rows of stopped
    // systems are skipped by the row-per-thread kernels while mask_rows is set), else null
    const int* rowseg = nullptr;
    const int* act = nullptr;
    // SELL-32 in quads with 16-bit offsets (sellq_kernel), for the FP32 passes in natural order; null
    // when the matrix is colour-grouped, uses the lane-group layout, or a slice's columns do not fit
    int* q_sptr = nullptr;
    int2* q_base = nullptr;
    uint2* q_col = nullptr;
    float4* q_val = nullptr;
    long q_padded = 0;
    std::vector<int> group_slice;   // colour c occupies slices [group_slice[c], group_slice[c+1])
    // CSR-vector layout (lanes > 0): CSR arrays and, for colour groups, the rows of each colour
    int lanes = 0;
    int* ptr = nullptr;
    int* rows = nullptr;
    std::vector<int> group_row;     // colour c: rows[group_row[c] .. group_row[c+1])
    int* d_group_row = nullptr;     // the same offsets on the device
    int* d_head = nullptr;          // per position of rows: (row, ptr[row], ptr[row + 1], 0)
    int max_group_rows = 0;         // rows of the largest colour
};

// Layout choice, from sweeps of every level of the 2.1M-dof elasticity hierarchy on GB300 in every
// layout (FP32 and FP64): one thread per row (SELL-32; long rows software-pipelined) for levels of
// 100k rows or more; a group of lanes per row for the small coarse levels, 8 lanes from 8k rows
// (enough rows to fill the GPU, several loads in flight per lane), wider groups below.
int csrv_lanes_for_shape(long n, double avg) {
    if (g_layout == 1) return 0;
    if (g_layout >= 3) return 4 << (g_layout - 3);
    if (g_layout == 0 && n >= 100000 && avg <= 256.0) return 0;
    if (avg < 8.0) return 4;
    if (n >= 8000) return 8;
    return avg >= 24.0 ? 16 : 8;
}

int csrv_lanes_for(const lina::Csr& c) {
    return csrv_lanes_for_shape(c.n, c.n > 0 ? double(c.nnz()) / c.n : 0.0);
}

// Host-side SELL-32 construction; `order` lists the rows per group (colour)
// and each group starts on a slice boundary.  Without groups the natural row
// order is used.
struct SellHost {
    std::vector<int> sptr{0}, col, rowmap;
    std::vector<double> val;
    std::vector<int> group_slice{0};
    std::vector<int> pos;  // SELL position of each CSR entry (-1: not stored)
};

// Padding entries repeat a column the row already uses (or column 0 for an
// empty row), so every gathered index lies inside the input vector.
SellHost make_sell(const lina::Csr& A, int ncols, const std::vector<std::vector<int>>* groups) {
    SellHost S;
    S.pos.assign(A.nnz(), -1);
    auto add_group = [&](const int* rows, int nr) {
        for (int base = 0; base < nr; base += 32) {
            int len = 0;
            for (int l = 0; l < 32 && base + l < nr; l++) {
                int r = rows ? rows[base + l] : base + l;
                len = std::max(len, A.ptr[r + 1] - A.ptr[r]);
            }
            const size_t off = S.col.size();
            S.col.resize(off + 32 * (size_t)len);
            S.val.resize(off + 32 * (size_t)len);
            for (int l = 0; l < 32; l++) {
                const bool valid = base + l < nr;
                const int r = valid ? (rows ? rows[base + l] : base + l) : -1;
                const int rl = valid ? A.ptr[r + 1] - A.ptr[r] : 0;
                int pad_col = 0;
                for (int k = 0; k < rl; k++)
                    if (A.col[A.ptr[r] + k] < ncols) {
                        pad_col = A.col[A.ptr[r] + k];
                        break;
                    }
                for (int k = 0; k < len; k++) {
                    const size_t q = off + 32 * (size_t)k + l;
                    if (k < rl && A.col[A.ptr[r] + k] < ncols) {
                        S.col[q] = A.col[A.ptr[r] + k];
                        S.val[q] = A.val[A.ptr[r] + k];
                        S.pos[A.ptr[r] + k] = (int)q;
                    } else {
                        // padding, or an explicit zero whose column lies outside the
                        // operand (the reference's (i, 0.0) placeholder of an empty row)
                        S.col[q] = pad_col;
                        S.val[q] = 0.0;
                    }
                }
                S.rowmap.push_back(r);
            }
            S.sptr.push_back((int)S.col.size());
        }
        S.group_slice.push_back((int)S.sptr.size() - 1);
    };
    if (groups) {
        for (const auto& g : *groups) add_group(g.data(), (int)g.size());
        return S;
    }
    // natural order: the slices are independent, built in parallel (the same layout as add_group)
    const int ns = (A.n + 31) / 32;
    std::vector<int> slen(ns, 0);
#pragma omp parallel for schedule(static)
    for (int sl = 0; sl < ns; sl++) {
        int len = 0;
        for (int r = 32 * sl; r < std::min(A.n, 32 * sl + 32); r++) len = std::max(len, A.ptr[r + 1] - A.ptr[r]);
        slen[sl] = len;
    }
    S.sptr.assign(ns + 1, 0);
    for (int sl = 0; sl < ns; sl++) S.sptr[sl + 1] = S.sptr[sl] + 32 * slen[sl];
    S.col.assign(S.sptr[ns], 0);
    S.val.assign(S.sptr[ns], 0.0);
    S.rowmap.assign(32 * (size_t)ns, -1);
#pragma omp parallel for schedule(static)
    for (int sl = 0; sl < ns; sl++) {
        const size_t off = S.sptr[sl];
        for (int l = 0; l < 32; l++) {
            const int r = 32 * sl + l;
            const bool valid = r < A.n;
            const int rl = valid ? A.ptr[r + 1] - A.ptr[r] : 0;
            int pad_col = 0;
            for (int k = 0; k < rl; k++)
                if (A.col[A.ptr[r] + k] < ncols) {
                    pad_col = A.col[A.ptr[r] + k];
                    break;
                }
            for (int k = 0; k < slen[sl]; k++) {
                const size_t q = off + 32 * (size_t)k + l;
                if (k < rl && A.col[A.ptr[r] + k] < ncols) {
                    S.col[q] = A.col[A.ptr[r] + k];
                    S.val[q] = A.val[A.ptr[r] + k];
                    S.pos[A.ptr[r] + k] = (int)q;
                } else {
                    S.col[q] = pad_col;
                    S.val[q] = 0.0;
                }
            }
            S.rowmap[32 * (size_t)sl + l] = valid ? r : -1;
        }
    }
    S.group_slice.push_back(ns);
    return S;
}

// 16-bit column offsets of a SELL-32 matrix (see sell_kernel): per slice, base.x = the smallest
// column of its rows, base.y = the smallest column beyond base.x + 32767 (base.x if none).  Fails
// (false) if some slice has a column beyond both windows.  Entries of padding positions (rows past
// the end, or -1 in the colour order) are never read and hold 0.
// The quad layout of sellq_kernel for a natural-order matrix: pos[k] receives each CSR entry's stored
// position (-1 for an explicit zero whose column lies outside the operand, stored as padding).  False
// when some slice's columns do not fit two windows of 32,768.
struct QuadHost {
    std::vector<int> sptr;
    std::vector<int2> base;
    std::vector<unsigned short> col;  // four per group
    std::vector<float> val;
    std::vector<int> pos;
};

bool make_quads(const lina::Csr& A, int ncols, QuadHost& Q) {
    const int n = A.n, ns = (n + 31) / 32;
    Q.sptr.assign(ns + 1, 0);
    for (int s = 0; s < ns; s++) {
        int len = 0;
        for (int l = 0; l < 32 && 32 * s + l < n; l++) len = std::max(len, A.ptr[32 * s + l + 1] - A.ptr[32 * s + l]);
        len = (len + 3) / 4 * 4;
        if ((long)Q.sptr[s] + 32L * len > (long)INT_MAX) return false;
        Q.sptr[s + 1] = Q.sptr[s] + 32 * len;
    }
    const size_t total = (size_t)Q.sptr[ns];
    Q.col.assign(total, 0);
    Q.val.assign(total, 0.f);
    Q.base.assign(ns, make_int2(0, 0));
    Q.pos.assign(A.nnz(), -1);
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int s = 0; s < ns; s++) {
        const size_t p0 = (size_t)Q.sptr[s];
        const int len = (Q.sptr[s + 1] - Q.sptr[s]) / 32;
        // the two 16-bit windows of the slice, from its rows' columns inside the operand
        int lo = INT_MAX, hi = INT_MAX;
        for (int l = 0; l < 32 && 32 * s + l < n; l++) {
            const int r = 32 * s + l;
            for (int p = A.ptr[r]; p < A.ptr[r + 1]; p++)
                if (A.col[p] < ncols) lo = std::min(lo, A.col[p]);
        }
        if (lo == INT_MAX) lo = 0;
        for (int l = 0; l < 32 && 32 * s + l < n; l++) {
            const int r = 32 * s + l;
            for (int p = A.ptr[r]; p < A.ptr[r + 1]; p++)
                if (A.col[p] < ncols && (long)A.col[p] - lo > 32767) hi = std::min(hi, A.col[p]);
        }
        if (hi == INT_MAX) hi = lo;
        Q.base[s] = make_int2(lo, hi);
        auto code = [&](int c, int& out) {
            if ((long)c - lo <= 32767) {
                out = c - lo;
                return true;
            }
            if (c >= hi && (long)c - hi <= 32767) {
                out = 0x8000 | (c - hi);
                return true;
            }
            return false;
        };
        for (int l = 0; l < 32; l++) {
            const int r = 32 * s + l;
            const bool valid = r < n;
            const int rl = valid ? A.ptr[r + 1] - A.ptr[r] : 0;
            int pad = lo;
            for (int k = 0; k < rl; k++)
                if (A.col[A.ptr[r] + k] < ncols) {
                    pad = A.col[A.ptr[r] + k];
                    break;
                }
            for (int k = 0; k < len; k++) {
                const size_t q = p0 + (size_t)128 * (k / 4) + 4 * (size_t)l + (k % 4);
                int c = pad;
                float v = 0.f;
                if (k < rl && A.col[A.ptr[r] + k] < ncols) {
                    c = A.col[A.ptr[r] + k];
                    v = (float)A.val[A.ptr[r] + k];
                    Q.pos[A.ptr[r] + k] = (int)q;
                }
                int e = 0;
                if (!code(c, e)) bad = 1;
                Q.col[q] = (unsigned short)e;
                Q.val[q] = v;
            }
        }
    }
    return !bad;
}

bool encode_sell16(const SellHost& S, int nrows, std::vector<unsigned short>& c16, std::vector<int2>& base) {
    const int ns = (int)S.sptr.size() - 1;
    c16.assign(S.col.size(), 0);
    base.assign(ns, make_int2(0, 0));
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int sl = 0; sl < ns; sl++) {
        const long p0 = S.sptr[sl], len = (S.sptr[sl + 1] - p0) / 32;
        auto valid = [&](int l) {
            const int r = S.rowmap[32 * (size_t)sl + l];
            return r >= 0 && r < nrows;
        };
        int lo = INT_MAX, hi2 = INT_MAX;
        for (int l = 0; l < 32; l++)
            if (valid(l))
                for (long k = 0; k < len; k++) lo = std::min(lo, S.col[p0 + 32 * k + l]);
        if (lo == INT_MAX) continue;
        for (int l = 0; l < 32; l++)
            if (valid(l))
                for (long k = 0; k < len; k++) {
                    const int c = S.col[p0 + 32 * k + l];
                    if ((long)c - lo > 32767) hi2 = std::min(hi2, c);
                }
        if (hi2 == INT_MAX) hi2 = lo;
        base[sl] = make_int2(lo, hi2);
        for (int l = 0; l < 32; l++)
            if (valid(l))
                for (long k = 0; k < len; k++) {
                    const size_t q = p0 + 32 * k + l;
                    const long c = S.col[q];
                    if (c - lo <= 32767)
                        c16[q] = (unsigned short)(c - lo);
                    else if (c >= hi2 && c - hi2 <= 32767)
                        c16[q] = (unsigned short)(0x8000 | (c - hi2));
                    else
                        bad = 1;
                }
    }
    return !bad;
}

struct DLevel {
    int n = 0;
    DCsr A, P, R;
    DCsr Acol;  // rows grouped by colour (multicolour SOR)
    // a level of independent systems (segmented batch): the cluster-fused multicolour-SOR step runs one
    // cluster per group of whole systems (ngroups > 0)
    int ngroups = 0, max_group_rows = 0;
    FusedGroup* d_groups = nullptr;
    // the staged fused step (stage_k blocks, 0: none); images as StagedPlan describes them
    int stage_k = 0, stage_ints = 0, stage_nvals = 0, stage_pslots = 0;
    int stage_o_row = 0, stage_o_off = 0, stage_o_col = 0, stage_o_dinv = 0;
    int* stage_int = nullptr;
    int* stage_src = nullptr;  // per value slot: the CSR entry, -2 - row for 1/a_ii, -1 padding
    double* stage_v64 = nullptr;
    float* stage_v32 = nullptr;
    double* dinv64 = nullptr;
    float* dinv32 = nullptr;
    int ncolours = 0;
    double *x64 = nullptr, *t64 = nullptr, *b64 = nullptr, *r64 = nullptr;
    float *x32 = nullptr, *t32 = nullptr, *b32 = nullptr, *r32 = nullptr;
};

// every non-CSR launch goes through here so that the library can report how many
// kernels it issued
// Every kernel of this file starts with pdl_wait(), so it may be launched with programmatic stream
// serialisation (g_pdl, default on): its blocks start while the previous kernel drains, which hides most
// of the launch gap between the many short kernels of a V-cycle.
template <typename... KA, typename... A>
void launch(void (*k)(KA...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A... a) {
    g_launches++;
    if (g_pdl) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k, static_cast<KA>(a)...);
    } else {
        k<<<grid, block, smem, st>>>(a...);
    }
}

template <typename... KA, typename... A>
void go(void (*k)(KA...), int grid, cudaStream_t st, A... a) {
    launch(k, dim3(grid), dim3(kThreads), 0, st, a...);
}

int grid_for(long items, int per_block) {
    long g = (items + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > kGridCap) g = kGridCap;
    return (int)g;
}

int grid_red(long items) {
    long g = (items + kThreads - 1) / kThreads;
    if (g < 1) g = 1;
    if (g > kReduceGrid) g = kReduceGrid;
    return (int)g;
}

}  // namespace

struct lina_gpu_amg {
    lina::HostHierarchy host;
    lina_gpu_amg_options opt{};
    int depth = 0;
    std::vector<DLevel> lv;
    // coarsest dense block
    int cm = 0;
    int* c_brows = nullptr;
    int* c_inblock = nullptr;
    int* c_blockpos = nullptr;
    double* c_inv = nullptr;
    double* c_dginv = nullptr;
    double* c_bblk = nullptr;
    int *c_rblk = nullptr, *c_boff = nullptr;  // block-diagonal coarsest level (else null)
    long* c_ioff = nullptr;
    // finest-level extras
    double* isoinv = nullptr;  // 1/a for isolated rows of the finest level, 0 elsewhere
    double* signs = nullptr;   // only when make_positive_diag flipped a row
    DCsr Aorig;                // unflipped finest matrix when signs exist (Krylov SpMV)
    bool has_signs = false;
    bool host_only = false;
    // segmented batch: per level, the rows of the largest system's level (layout choice), else empty
    std::vector<long> seg_max_rows;
    std::vector<std::vector<int>> seg_off;  // per level, the first row of each system (and the end)
    long lanes_rows = 0;
    // layout autotuning: on for this hierarchy, the lanes per row forced on the next uploads (-1: the
    // rule), and per level the choice made (-1: not tuned), kept for later re-uploads (recompute)
    bool autotune = false;
    bool mask_rows = false;  // the segmented iteration: skip the rows of systems that have stopped
    int force_lanes = -1;
    std::vector<int> tuned_lanes;
    // lina_gpu_amg_recompute: per level, where each CSR entry of A sits in the device layouts (natural,
    // quads, colour-grouped) and a fingerprint of A's pattern, kept from the first recompute on so that
    // later ones with the same patterns only move values
    struct LevelMaps {
        int *posA = nullptr, *posQ = nullptr, *posC = nullptr;
        uint64_t pattern = 0;
        long nnz = 0;
    };
    std::vector<LevelMaps> rmaps;
    bool keep_maps = false;
    double* rstage = nullptr;  // staging for a level's new values
    long rstage_n = 0;
    int* rerr = nullptr;       // error word of the device coarse inverse
    std::vector<int> c_block_rows;  // the coarse block rows of the uploaded coarse solver
    int timed_level = 0;       // level whose smoother sweeps LINA_PCG_TIME_KERNELS times (most entries)
    // maps for lina_gpu_amg_update_values (built on first use, finest level)
    bool upd_built = false;
    long upd_nnz = 0;
    int *upd_posA = nullptr, *upd_posAcol = nullptr, *upd_diagpos = nullptr, *upd_ptr = nullptr;
    int* upd_posQ = nullptr;  // quad-layout positions of the finest matrix's entries (when it has that layout)
    unsigned char* upd_isolated = nullptr;
    double* upd_val = nullptr;  // staging for host values
    // Krylov work
    double *kr = nullptr, *kz = nullptr, *kp = nullptr, *kq = nullptr, *kx = nullptr, *kb = nullptr,
           *kt = nullptr;
    float* kz32 = nullptr;
    // truncated flexible CG: directions kept (0: the precision's default), and their rings
    int fcg_m = 0;
    int hist_m = 0;  // slots allocated in kph / kqh
    double *kph = nullptr, *kqh = nullptr;
    double* partials = nullptr;
    unsigned* ticket = nullptr;
    KScalars* sc = nullptr;
    KScalars* sc_host = nullptr;
    double* hscal = nullptr;  // device scalar for normalisation
    cudaStream_t stream = nullptr;
    long dev_bytes = 0;
    std::vector<void*> allocations;
    // CUDA graph of one PCG iteration inside a device-side while loop
    cudaGraphExec_t gexec = nullptr;
    int g_prec = -1, g_smoother = -1, g_flexible = -1, g_history = -1;
    double g_omega = 0.0;
    long g_kernels = 0;  // kernels per captured iteration
    void drop_graph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
        g_prec = -1;
    }
    // smoother timing
    cudaEvent_t tm0 = nullptr, tm1 = nullptr;
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    int ev_used = 0;

    ~lina_gpu_amg() {
        drop_graph();
        for (void* p : allocations) cudaFree(p);
        if (sc_host) cudaFreeHost(sc_host);
        for (auto e : ev_pool) cudaEventDestroy(e);
        if (tm0) cudaEventDestroy(tm0);
        if (tm1) cudaEventDestroy(tm1);
        if (stream) cudaStreamDestroy(stream);
    }

    template <typename T>
    int alloc(T** p, size_t count) {
        if (count == 0) count = 1;
        if (g_mem_limit > 0 && dev_bytes + (long)(count * sizeof(T)) > g_mem_limit) {
            set_err("cudaMalloc(%zu bytes) refused: the handle's device-memory limit of %ld bytes "
                    "(lina_gpu_set_device_memory_limit) would be exceeded", count * sizeof(T), g_mem_limit);
            *p = nullptr;
            return LINA_GPU_ECUDA;
        }
        cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
        if (e != cudaSuccess) {
            set_err("cudaMalloc(%zu bytes) failed: %s", count * sizeof(T), cudaGetErrorString(e));
            *p = nullptr;
            return LINA_GPU_ECUDA;
        }
        allocations.push_back((void*)*p);
        dev_bytes += (long)(count * sizeof(T));
        return 0;
    }
    template <typename T>
    int upload(T** p, const T* src, size_t count) {
        int rc = alloc(p, count);
        if (rc) return rc;
        if (count) CK(cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, stream));
        return 0;
    }
    // pos_out (optional): the stored position of every CSR entry (-1: not stored), empty for the
    // lane-group layout, whose positions are the CSR order
    int upload_csr(DCsr& d, const lina::Csr& c, const std::vector<std::vector<int>>* groups = nullptr,
                   std::vector<int>* pos_out = nullptr, std::vector<int>* qpos_out = nullptr) {
        d = DCsr();
        d.n = c.n;
        d.ncols = c.ncols;
        d.nnz = c.nnz();
        if (c.nnz() > (long)INT_MAX / 2) {
            set_err("matrix too large for 32-bit SELL offsets");
            return LINA_GPU_EINVAL;
        }
        const int ncols = c.ncols > 0 ? c.ncols : c.n;
        long bad = -1;
#pragma omp parallel for schedule(static) reduction(max : bad)
        for (long k = 0; k < (long)c.col.size(); k++)
            if (c.col[k] < 0 || (c.col[k] >= ncols && c.val[k] != 0.0)) bad = std::max(bad, k);
        if (bad >= 0) {
            set_err("matrix entry with column %d outside [0, %d)", c.col[bad], ncols);
            return LINA_GPU_EINVAL;
        }
        // a level of a segmented batch takes the layout of its largest system's level (lanes_rows rows):
        // concatenated small levels keep the lane groups their long rows need; an autotuned level the
        // layout measured fastest (force_lanes)
        d.lanes = force_lanes >= 0 ? force_lanes
                  : lanes_rows > 0 ? csrv_lanes_for_shape(std::min<long>(lanes_rows, c.n), c.n > 0 ? double(c.nnz()) / c.n : 0.0)
                                   : csrv_lanes_for(c);
        if (d.lanes > 0) {
            // CSR-vector: sanitise placeholder columns outside the operand, keep the CSR arrays
            std::vector<int> colc(c.col);
            for (size_t k = 0; k < colc.size(); k++)
                if (colc[k] >= ncols) colc[k] = 0;  // value is 0.0 (checked above)
            std::vector<float> v32(c.val.begin(), c.val.end());
            int rc;
            if ((rc = upload(&d.ptr, c.ptr.data(), c.ptr.size()))) return rc;
            if ((rc = upload(&d.col, colc.data(), colc.size()))) return rc;
            if ((rc = upload(&d.v64, c.val.data(), c.val.size()))) return rc;
            if ((rc = upload(&d.v32, v32.data(), v32.size()))) return rc;
            d.padded = c.nnz();
            d.group_row.assign(1, 0);
            if (groups) {
                std::vector<int> all;
                for (const auto& g : *groups) {
                    all.insert(all.end(), g.begin(), g.end());
                    d.group_row.push_back((int)all.size());
                }
                if ((rc = upload(&d.rows, all.data(), all.size()))) return rc;
                if ((rc = upload(&d.d_group_row, d.group_row.data(), d.group_row.size()))) return rc;
                std::vector<int> head(4 * all.size(), 0);
                for (size_t g = 0; g < all.size(); g++) {
                    head[4 * g] = all[g];
                    head[4 * g + 1] = c.ptr[all[g]];
                    head[4 * g + 2] = c.ptr[all[g] + 1];
                }
                if ((rc = upload(&d.d_head, head.data(), head.size()))) return rc;
                for (size_t k = 0; k + 1 < d.group_row.size(); k++)
                    d.max_group_rows = std::max(d.max_group_rows, d.group_row[k + 1] - d.group_row[k]);
            } else {
                d.group_row.push_back(c.n);
            }
            d.group_slice.assign(1, 0);
            // mid-size levels: FP32 passes in natural order read the quad layout (measured on the 34k-row
            // level of the 2.1M-dof elasticity hierarchy: 8-10 us per sweep against 12 us in lane groups)
            if (!groups && c.n >= kQuadMinRows && (rc = upload_quads(d, c, ncols, qpos_out))) return rc;
            return cudaStreamSynchronize(stream) == cudaSuccess ? 0 : LINA_GPU_ECUDA;
        }
        SellHost S = make_sell(c, ncols, groups);
        if (pos_out) pos_out->swap(S.pos);
        d.long_rows = c.n > 0 && double(c.nnz()) / c.n >= 24.0;
        if (S.col.size() > (size_t)INT_MAX) {
            set_err("padded matrix too large for 32-bit SELL offsets");
            return LINA_GPU_EINVAL;
        }
        d.padded = (long)S.col.size();
        d.npos = (int)S.rowmap.size();
        d.group_slice = S.group_slice;
        std::vector<float> v32(S.val.size());
#pragma omp parallel for schedule(static)
        for (long k = 0; k < (long)S.val.size(); k++) v32[k] = (float)S.val[k];
        int rc;
        if ((rc = upload(&d.sptr, S.sptr.data(), S.sptr.size()))) return rc;
        if ((rc = upload(&d.col, S.col.data(), S.col.size()))) return rc;
        // FP32 passes over long rows read 16-bit columns where the slices fit (measured on the 2.1M-dof
        // elasticity hierarchy: 8-17 % faster sweeps on its long-row levels; no gain on the short
        // rows of the finest level, and none in FP64, which keeps int columns)
        std::vector<unsigned short> c16;
        std::vector<int2> sbase;
        if (g_sell_bits == 16 && d.long_rows && encode_sell16(S, c.n, c16, sbase)) {
            if ((rc = upload(&d.col16, c16.data(), c16.size()))) return rc;
            if ((rc = upload(&d.sbase, sbase.data(), sbase.size()))) return rc;
        }
        if ((rc = upload(&d.v64, S.val.data(), S.val.size()))) return rc;
        if ((rc = upload(&d.v32, v32.data(), v32.size()))) return rc;
        if (groups) {
            if ((rc = upload(&d.rowmap, S.rowmap.data(), S.rowmap.size()))) return rc;
        }
        // FP32 passes in natural order read the quad layout (sellq_kernel) where the columns fit 16 bits
        if (!groups && (rc = upload_quads(d, c, ncols, qpos_out))) return rc;
        // the host copies must outlive the asynchronous uploads
        return cudaStreamSynchronize(stream) == cudaSuccess ? 0 : LINA_GPU_ECUDA;
    }

    // the quad layout of a natural-order matrix, where enabled and its columns fit 16-bit offsets (the
    // matrix keeps its other layout for FP64 passes); synchronises before the host copy is released
    static constexpr int kQuadMinRows = 20000;
    int upload_quads(DCsr& d, const lina::Csr& c, int ncols, std::vector<int>* qpos_out) {
        if (g_sell_bits != 16 || !g_quads) return 0;
        QuadHost Q;
        if (!make_quads(c, ncols, Q)) return 0;
        int rc;
        if ((rc = upload(&d.q_sptr, Q.sptr.data(), Q.sptr.size()))) return rc;
        if ((rc = upload(&d.q_base, Q.base.data(), Q.base.size()))) return rc;
        if ((rc = alloc(&d.q_col, Q.col.size() / 4))) return rc;
        if ((rc = alloc(&d.q_val, Q.val.size() / 4))) return rc;
        CK(cudaMemcpyAsync(d.q_col, Q.col.data(), Q.col.size() * sizeof(unsigned short), cudaMemcpyHostToDevice,
                           stream));
        CK(cudaMemcpyAsync(d.q_val, Q.val.data(), Q.val.size() * sizeof(float), cudaMemcpyHostToDevice, stream));
        d.q_padded = (long)Q.val.size();
        if (qpos_out) qpos_out->swap(Q.pos);
        return cudaStreamSynchronize(stream) == cudaSuccess ? 0 : LINA_GPU_ECUDA;
    }

    // ------------------------------------------------------------ timing
    void ev_record_pair_start(cudaEvent_t* a) {
        if (ev_used + 2 > (int)ev_pool.size()) {
            for (int k = 0; k < 64; k++) {
                cudaEvent_t e;
                cudaEventCreate(&e);
                ev_pool.push_back(e);
            }
        }
        *a = ev_pool[ev_used];
        cudaEventRecord(*a, stream);
        ev_used += 1;
    }
    void ev_record_pair_end() {
        cudaEventRecord(ev_pool[ev_used], stream);
        ev_used += 1;
    }

    // ------------------------------------------------------------ kernels
    template <typename TV, typename TX, int MODE>
    void launch_sell_t(const DCsr& m, const TV* val, int slice0, int slice1, const TX* x, TX* y, const TX* b,
                       const TX* dinv, TX w, const TX* z) {
        const int npos = (slice1 - slice0) * 32;
        if (npos <= 0) return;
        int grid = (npos + kThreads - 1) / kThreads;
        if (MODE == M_DOT && grid > kMaxBlocks) grid = kMaxBlocks;
        g_launches++;
        const int* rm = m.rowmap ? m.rowmap + (size_t)slice0 * 32 : nullptr;
        // natural order: rows of this range are [32 slice0, n); colour order: the row map marks padding
        const int nrows = rm ? m.n : m.n - 32 * slice0;
        const int* sp = m.sptr + slice0;
        if constexpr (sizeof(TX) == 4 && (MODE == M_SPMV || MODE == M_RESID || MODE == M_JACOBI || MODE == M_ADD)) {
            if (m.q_val && !m.rowmap && slice0 == 0 && 32 * slice1 >= m.n) {
                g_launches--;  // counted by launch()
                launch(sellq_kernel<MODE>, dim3(grid), dim3(kThreads), 0, stream, m.n, (const int*)m.q_sptr,
                       (const int2*)m.q_base, (const uint2*)m.q_col, (const float4*)m.q_val, (const float*)x,
                       (float*)y, (const float*)b, (const float*)dinv, (float)w, (const float*)z,
                       mask_rows ? m.rowseg : (const int*)nullptr, m.act);
                return;
            }
        }
        g_launches--;  // counted by launch()
        const dim3 gd(grid), bd(kThreads);
        // row indices of a natural-order range start at 32 slice0; of the colour order, they are global
        const int* rseg = (mask_rows && m.rowseg) ? (rm ? m.rowseg : m.rowseg + (size_t)32 * slice0) : nullptr;
        if (sizeof(TX) == 4 && m.col16) {
            const int2* sb = m.sbase + slice0;
            if (m.long_rows)
                launch(sell_kernel<TV, TX, MODE, true, unsigned short>, gd, bd, 0, stream, npos, nrows, rm, sp, sb,
                       (const unsigned short*)m.col16, val, x, y, b, dinv, w, z, partials, ticket, sc, rseg, m.act);
            else
                launch(sell_kernel<TV, TX, MODE, false, unsigned short>, gd, bd, 0, stream, npos, nrows, rm, sp, sb,
                       (const unsigned short*)m.col16, val, x, y, b, dinv, w, z, partials, ticket, sc, rseg, m.act);
        } else if (m.long_rows) {
            launch(sell_kernel<TV, TX, MODE, true, int>, gd, bd, 0, stream, npos, nrows, rm, sp, (const int2*)nullptr,
                   (const int*)m.col, val, x, y, b, dinv, w, z, partials, ticket, sc, rseg, m.act);
        } else {
            launch(sell_kernel<TV, TX, MODE, false, int>, gd, bd, 0, stream, npos, nrows, rm, sp, (const int2*)nullptr,
                   (const int*)m.col, val, x, y, b, dinv, w, z, partials, ticket, sc, rseg, m.act);
        }
        if (MODE == M_DOT) launch(dot_finish_kernel, dim3(1), dim3(1024), 0, stream, grid, (const double*)partials, sc);
    }

    template <typename TV, typename TX, int MODE>
    void launch_csrv_t(const DCsr& m, const TV* val, int r0, int r1, const TX* x, TX* y, const TX* b,
                       const TX* dinv, TX w, const TX* z) {
        const int nrows = r1 - r0;
        if (nrows <= 0) return;
        if constexpr (sizeof(TX) == 4 && (MODE == M_SPMV || MODE == M_RESID || MODE == M_JACOBI || MODE == M_ADD)) {
            if (m.q_val && !m.rows && r0 == 0 && r1 == m.n) {
                const int grid = (((m.n + 31) / 32) * 32 + kThreads - 1) / kThreads;
                launch(sellq_kernel<MODE>, dim3(grid), dim3(kThreads), 0, stream, m.n, (const int*)m.q_sptr,
                       (const int2*)m.q_base, (const uint2*)m.q_col, (const float4*)m.q_val, (const float*)x,
                       (float*)y, (const float*)b, (const float*)dinv, (float)w, (const float*)z,
                       mask_rows ? m.rowseg : (const int*)nullptr, m.act);
                return;
            }
        }
        const int S = m.lanes;
        long grid = ((long)nrows * S + kThreads - 1) / kThreads;
        if (MODE == M_DOT && grid > kMaxBlocks) grid = kMaxBlocks;
        if (grid > (1L << 30)) grid = 1L << 30;
        const int* rl = m.rows ? m.rows + r0 : nullptr;
#define LINA_CSRV_CASE(SS)                                                                                       \
    case SS:                                                                                                     \
        launch(csrv_kernel<TV, TX, SS, MODE>, dim3((int)grid), dim3(kThreads), 0, stream, nrows, rl,              \
               (const int*)m.ptr, (const int*)m.col, val, x, y, b, dinv, w, z, partials, ticket, sc);             \
        break;
        switch (S) {
            LINA_CSRV_CASE(4)
            LINA_CSRV_CASE(8)
            LINA_CSRV_CASE(16)
            default:
                LINA_CSRV_CASE(32)
        }
#undef LINA_CSRV_CASE
        if (MODE == M_DOT) launch(dot_finish_kernel, dim3(1), dim3(1024), 0, stream, (int)grid, (const double*)partials, sc);
    }

    // all rows of m (natural order)
    template <typename TX, int MODE>
    void csr(const DCsr& m, const TX* x, TX* y, const TX* b = nullptr, const TX* dinv = nullptr, TX w = TX(0),
             const TX* z = nullptr) {
        if (m.lanes > 0) {
            if constexpr (sizeof(TX) == 8)
                launch_csrv_t<double, TX, MODE>(m, m.v64, 0, m.n, x, y, b, dinv, w, z);
            else
                launch_csrv_t<float, TX, MODE>(m, m.v32, 0, m.n, x, y, b, dinv, w, z);
            return;
        }
        const int ns = (int)m.group_slice.back();
        if constexpr (sizeof(TX) == 8)
            launch_sell_t<double, TX, MODE>(m, m.v64, 0, ns, x, y, b, dinv, w, z);
        else
            launch_sell_t<float, TX, MODE>(m, m.v32, 0, ns, x, y, b, dinv, w, z);
    }

    // the rows of colour c of a colour-grouped matrix
    template <typename TX, int MODE>
    void csr_group(const DCsr& m, int c, const TX* x, TX* y, const TX* b, const TX* dinv, TX w) {
        if (m.lanes > 0) {
            if constexpr (sizeof(TX) == 8)
                launch_csrv_t<double, TX, MODE>(m, m.v64, m.group_row[c], m.group_row[c + 1], x, y, b, dinv, w,
                                                nullptr);
            else
                launch_csrv_t<float, TX, MODE>(m, m.v32, m.group_row[c], m.group_row[c + 1], x, y, b, dinv, w,
                                               nullptr);
            return;
        }
        if constexpr (sizeof(TX) == 8)
            launch_sell_t<double, TX, MODE>(m, m.v64, m.group_slice[c], m.group_slice[c + 1], x, y, b, dinv, w,
                                            nullptr);
        else
            launch_sell_t<float, TX, MODE>(m, m.v32, m.group_slice[c], m.group_slice[c + 1], x, y, b, dinv, w,
                                           nullptr);
    }

    // ------------------------------------------------------------ V-cycle
    template <typename TX>
    TX* lvx(DLevel& L, int which) {  // 0 x, 1 t, 2 b, 3 r
        if constexpr (sizeof(TX) == 8) {
            double* v[4] = {L.x64, L.t64, L.b64, L.r64};
            return v[which];
        } else {
            float* v[4] = {L.x32, L.t32, L.b32, L.r32};
            return v[which];
        }
    }
    template <typename TX>
    const TX* lvdinv(DLevel& L) {
        if constexpr (sizeof(TX) == 8)
            return L.dinv64;
        else
            return L.dinv32;
    }

    template <typename TX>
    void coarse_solve(const TX* b, TX* x) {
        const int n = lv[0].n;
        go(coarse_gather_kernel<TX>, grid_for(n, kThreads), stream, n, b, c_inblock, c_blockpos,
                                                                                 c_dginv, c_bblk, x);
        if (cm > 0)
            go(coarse_gemv_kernel<TX>, grid_for((long)cm * 32, kThreads), stream, cm, (const double*)c_inv,
               (const double*)c_bblk, (const int*)c_brows, x, (const int*)c_rblk, (const int*)c_boff,
               (const long*)c_ioff);
    }

    // pre-smoothing from the zero guess (plus the isolated-row fix on the finest level)
    template <typename TB, typename TX>
    void presmooth(DLevel& L, int nu, const TB* bin, const double* sign, const double* iso, TX* b, TX* x,
                   bool time_it) {
        const TX w = TX(opt.omega);
        const TX* dinv = lvdinv<TX>(L);
        TX* t = lvx<TX>(L, 1);
        TX* bout = ((const void*)bin == (const void*)b) ? nullptr : b;
        if (opt.smoother == LINA_SMOOTHER_JACOBI && nu > 0) {
            TX* cur = ((nu - 1) % 2 == 0) ? x : t;
            go(jacobi_first_kernel<TB, TX>, grid_for(L.n, kThreads), stream, L.n, bin, sign, dinv,
                                                                                           iso, w, cur, bout);
            for (int k = 1; k < nu; k++) {
                TX* nxt = (cur == x) ? t : x;
                cudaEvent_t e0;
                if (time_it) ev_record_pair_start(&e0);
                csr<TX, M_JACOBI>(L.A, cur, nxt, b, dinv, w);
                if (time_it) ev_record_pair_end();
                cur = nxt;
            }
        } else {
            go(init_x_kernel<TB, TX>, grid_for(L.n, kThreads), stream, L.n, bin, sign, iso, x, bout);
            for (int k = 0; k < nu; k++) sor_sweep(L, b, x, time_it);
        }
    }

    template <typename TX>
    void sor_sweep(DLevel& L, const TX* b, TX* x, bool time_it) {
        const TX w = TX(opt.omega);
        for (int c = 0; c < L.ncolours; c++) {
            cudaEvent_t e0;
            if (time_it) ev_record_pair_start(&e0);
            csr_group<TX, M_SOR>(L.Acol, c, x, x, b, lvdinv<TX>(L), w);
            if (time_it) ev_record_pair_end();
        }
    }

    // post-smoothing after the coarse correction x += P e; result ends in x
    template <typename TX>
    void correct_and_postsmooth(int l, DLevel& L, int nu, const TX* b, TX* x, const TX* e, bool time_it) {
        const TX w = TX(opt.omega);
        const TX* dinv = lvdinv<TX>(L);
        TX* t = lvx<TX>(L, 1);
        if (opt.smoother == LINA_SMOOTHER_JACOBI) {
            TX* cur = (nu % 2 == 0) ? x : t;
            csr<TX, M_ADD>(L.P, e, cur, nullptr, nullptr, TX(0), x);
            for (int k = 0; k < nu; k++) {
                TX* nxt = (cur == x) ? t : x;
                cudaEvent_t e0;
                if (time_it) ev_record_pair_start(&e0);
                csr<TX, M_JACOBI>(L.A, cur, nxt, b, dinv, w);
                if (time_it) ev_record_pair_end();
                cur = nxt;
            }
        } else {
            csr<TX, M_ADD>(L.P, e, x, nullptr, nullptr, TX(0), x);
            for (int k = 0; k < nu; k++) sor_sweep(L, b, x, time_it);
        }
        (void)l;
    }

    template <typename TX>
    void vcycle_level(int l, const TX* b, TX* x, bool time_it) {
        if (l == 0) {
            coarse_solve<TX>(b, x);
            return;
        }
        DLevel& L = lv[l];
        const int nu = (opt.coarsening == LINA_AGGRESSIVE && l == depth - 1) ? opt.aggr_smoothing_iterations
                                                                             : opt.smoothing_iterations;
        if (fusable(L, time_it && l == timed_level)) {
            DLevel& C = lv[l - 1];
            launch_fused<TX, true>(L, C, nu, b, x, nullptr);
            vcycle_level<TX>(l - 1, lvx<TX>(C, 2), lvx<TX>(C, 0), time_it);
            launch_fused<TX, false>(L, C, nu, b, x, lvx<TX>(C, 0));
            return;
        }
        presmooth<TX, TX>(L, nu, b, nullptr, nullptr, const_cast<TX*>(b), x, time_it && l == timed_level);
        run_rest<TX>(l, L, nu, b, x, time_it);
    }

    // an interior level whose multicolour-SOR step runs as one cluster launch (a copy of its x fits a
    // block's shared memory)
    bool fusable(const DLevel& L, bool timed) const {
        const long copy_bytes = (long)L.n * (opt.precision == LINA_PREC_MIXED ? 4 : 8);
        if (opt.smoother == LINA_SMOOTHER_JACOBI)  // two copies of x (the sweeps alternate)
            return g_fused_rows > 0 && g_fused_jacobi_entries > 0 && !timed && L.n <= g_fused_rows &&
                   L.A.nnz <= g_fused_jacobi_entries && 2 * copy_bytes <= kFusedSmemMax && L.A.lanes > 0 &&
                   L.R.lanes > 0 && L.P.lanes > 0;
        const bool whole = L.n <= g_fused_rows && copy_bytes <= kFusedSmemMax;
        const bool grouped = L.ngroups > 0 && L.max_group_rows <= g_fused_rows &&
                             (long)L.max_group_rows * (opt.precision == LINA_PREC_MIXED ? 4 : 8) <= kFusedSmemMax;
        return g_fused_rows > 0 && opt.smoother == LINA_SMOOTHER_MC_SOR && !timed && (whole || grouped) &&
               L.ncolours > 0 && L.Acol.lanes > 0 && L.Acol.d_group_row && L.Acol.d_head && L.A.lanes > 0 &&
               L.R.lanes > 0 && L.P.lanes > 0;
    }

    template <typename TX, bool PRE>
    void launch_fused(DLevel& L, DLevel& C, int nu, const TX* b, TX* x, const TX* e) {
        if (opt.smoother == LINA_SMOOTHER_JACOBI)
            launch_fused_as<TX, PRE, true>(L, C, nu, b, x, e);
        else
            launch_fused_as<TX, PRE, false>(L, C, nu, b, x, e);
    }

    template <typename TX, bool PRE, bool JAC>
    void launch_fused_as(DLevel& L, DLevel& C, int nu, const TX* b, TX* x, const TX* e) {
        FusedStep st;
        st.n = L.n;
        st.nc = C.n;
        st.ncolours = L.ncolours;
        st.nu = nu;
        st.sS = L.Acol.lanes;
        st.aS = L.A.lanes;
        st.rS = L.R.lanes;
        st.pS = L.P.lanes;
        st.sptr = L.Acol.ptr;
        st.scol = L.Acol.col;
        st.srows = L.Acol.rows;
        st.sgroup = L.Acol.d_group_row;
        st.shead = reinterpret_cast<const int4*>(L.Acol.d_head);
        st.aptr = L.A.ptr;
        st.acol = L.A.col;
        st.rptr = L.R.ptr;
        st.rcol = L.R.col;
        st.pptr = L.P.ptr;
        st.pcol = L.P.col;
        if constexpr (sizeof(TX) == 8) {
            st.sval = L.Acol.v64;
            st.aval = L.A.v64;
            st.rval = L.R.v64;
            st.pval = L.P.v64;
        } else {
            st.sval = L.Acol.v32;
            st.aval = L.A.v32;
            st.rval = L.R.v32;
            st.pval = L.P.v32;
        }
        st.dinv = lvdinv<TX>(L);
        st.b = b;
        st.e = e;
        st.x = x;
        st.r = lvx<TX>(L, 3);
        st.cb = lvx<TX>(C, 2);
        st.w = opt.omega;
        if (!JAC && L.stage_k > 0 && !(L.ngroups > 0 && L.n > g_fused_rows) &&
            L.stage_k <= staged_cluster_max<TX, PRE>()) {
            launch_staged<TX, PRE>(L, st);
            return;
        }
        const int K = fused_blocks<TX, PRE, JAC>();
        // whole systems in groups, one cluster each, where the level is too large for one cluster
        const bool grouped = !JAC && L.ngroups > 0 && L.n > g_fused_rows;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(K * (grouped ? L.ngroups : 1));
        cfg.blockDim = dim3(kFuseThreads);
        cfg.dynamicSmemBytes = (size_t)(JAC ? 2 : 1) * (grouped ? L.max_group_rows : L.n) * sizeof(TX);
        cfg.stream = stream;
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = K;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = g_pdl ? 2 : 1;
        g_launches++;
        cudaLaunchKernelEx(&cfg, fused_step_kernel<TX, PRE, JAC>, st,
                           grouped ? (const FusedGroup*)L.d_groups : (const FusedGroup*)nullptr);
    }

    // the staged step of a level: one cluster of its plan's blocks (see staged_step_kernel)
    template <typename TX, bool PRE>
    void launch_staged(const DLevel& L, const FusedStep& st) {
        StagedPlan sp;
        sp.img = L.stage_int;
        sp.vals = sizeof(TX) == 8 ? (const void*)L.stage_v64 : (const void*)L.stage_v32;
        sp.ints = L.stage_ints;
        sp.nvals = L.stage_nvals;
        sp.pslots = L.stage_pslots;
        sp.o_row = L.stage_o_row;
        sp.o_off = L.stage_o_off;
        sp.o_col = L.stage_o_col;
        sp.o_dinv = L.stage_o_dinv;
        sp.xbytes = (int)(((long)L.n * sizeof(TX) + 15) / 16 * 16);
        const int K = L.stage_k;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(K);
        cfg.blockDim = dim3(kFuseThreads);
        cfg.dynamicSmemBytes =
            (size_t)sp.xbytes + (size_t)(sp.nvals + sp.pslots) * sizeof(TX) + (size_t)sp.ints * sizeof(int);
        cfg.stream = stream;
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = K;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = g_pdl ? 2 : 1;
        g_launches++;
        cudaLaunchKernelEx(&cfg, staged_step_kernel<TX, PRE>, st, sp);
    }

    // the largest cluster of staged steps the GPU schedules with a full block of shared memory (16 where
    // it allows non-portable clusters, else 8)
    template <typename TX, bool PRE>
    static int staged_cluster_max() {
        static int k = 0;
        if (k == 0) {
            k = 8;
            cudaFuncSetAttribute(staged_step_kernel<TX, PRE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kStagedSmemMax);
            if (cudaFuncSetAttribute(staged_step_kernel<TX, PRE>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess) {
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(16);
                cfg.blockDim = dim3(kFuseThreads);
                cfg.dynamicSmemBytes = kStagedSmemMax;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = 16;
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                int nclusters = 0;
                if (cudaOccupancyMaxActiveClusters(&nclusters, staged_step_kernel<TX, PRE>, &cfg) == cudaSuccess &&
                    nclusters > 0)
                    k = 16;
            }
            cudaGetLastError();  // a refused attribute or query leaves no error behind
        }
        return k;
    }

    // blocks per cluster of an unstaged fused step: the largest cluster the GPU schedules, or fewer with
    // LINA_FUSED_CLUSTER (1, 2, 4 or 8)
    template <typename TX, bool PRE, bool JAC>
    static int fused_blocks() {
        const int kmax = fused_cluster_size<TX, PRE, JAC>();
        static int forced = -1;
        if (forced < 0) {
            const char* env = getenv("LINA_FUSED_CLUSTER");
            const int v = env ? atoi(env) : 0;
            forced = (v == 1 || v == 2 || v == 4 || v == 8 || v == 16) ? v : 0;
        }
        return forced > 0 ? std::min(forced, kmax) : kmax;
    }

    // 16 blocks per cluster where the GPU schedules such clusters, else the portable 8.  Measured on the
    // batch workload's 24-system sample: 16 blocks 3 % faster in total (the large elasticity systems
    // gain, the 10k-row ones lose 2 %).
    template <typename TX, bool PRE, bool JAC>
    static int fused_cluster_size() {
        static int k = 0;
        if (k == 0) {
            k = 8;
            cudaFuncSetAttribute(fused_step_kernel<TX, PRE, JAC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kFusedSmemMax);
            if (cudaFuncSetAttribute(fused_step_kernel<TX, PRE, JAC>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess) {
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(16);
                cfg.blockDim = dim3(kFuseThreads);
                cfg.dynamicSmemBytes = kFusedSmemMax;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = 16;
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                int nclusters = 0;
                if (cudaOccupancyMaxActiveClusters(&nclusters, fused_step_kernel<TX, PRE, JAC>, &cfg) == cudaSuccess &&
                    nclusters > 0)
                    k = 16;
            }
            cudaGetLastError();  // a refused attribute or query leaves no error behind
        }
        return k;
    }

    template <typename TX>
    void run_rest(int l, DLevel& L, int nu, const TX* b, TX* x, bool time_it) {
        TX* r = lvx<TX>(L, 3);
        DLevel& C = lv[l - 1];
        TX* cb = lvx<TX>(C, 2);
        TX* cx = lvx<TX>(C, 0);
        csr<TX, M_RESID>(L.A, x, r, b);
        csr<TX, M_SPMV>(L.R, r, cb);
        vcycle_level<TX>(l - 1, cb, cx, time_it);
        correct_and_postsmooth<TX>(l, L, nu, b, x, cx, time_it && l == timed_level);
    }

    // nu smoothing sweeps from the current x (not from zero); the result ends in x
    template <typename TX>
    void smooth_warm(DLevel& L, int nu, const TX* b, TX* x) {
        if (opt.smoother == LINA_SMOOTHER_JACOBI) {
            TX* t = lvx<TX>(L, 1);
            TX* cur = x;
            for (int k = 0; k < nu; k++) {
                TX* nxt = (cur == x) ? t : x;
                csr<TX, M_JACOBI>(L.A, cur, nxt, b, lvdinv<TX>(L), TX(opt.omega));
                cur = nxt;
            }
            if (cur != x) cudaMemcpyAsync(x, cur, (size_t)L.n * sizeof(TX), cudaMemcpyDeviceToDevice, stream);
        } else {
            for (int k = 0; k < nu; k++) sor_sweep(L, b, x, false);
        }
    }

    // Full multigrid (FMG_recursive / AMG_full_multigrid, LinA/Multigrid.c:1582-1611): the right-hand
    // side restricted to every level, the coarsest level solved, then on each finer level the
    // prolongated coarse solution improved by one V-cycle that starts from it.  F is the finest
    // right-hand side (signs applied, FP64 on the device); the result goes to X (FP64).
    template <typename TX>
    void fmg(const double* F, double* X) {
        const int f = depth - 1;
        TX* bf = lvx<TX>(lv[f], 2);
        const int gf = grid_for(lv[f].n, kThreads);
        go(convert_kernel<double, TX>, gf, stream, lv[f].n, F, bf);
        for (int l = f; l > 0; l--) csr<TX, M_SPMV>(lv[l].R, lvx<TX>(lv[l], 2), lvx<TX>(lv[l - 1], 2));
        coarse_solve<TX>(lvx<TX>(lv[0], 2), lvx<TX>(lv[0], 0));
        for (int l = 1; l <= f; l++) {
            DLevel& L = lv[l];
            TX* x = lvx<TX>(L, 0);
            const TX* b = lvx<TX>(L, 2);
            csr<TX, M_SPMV>(L.P, lvx<TX>(lv[l - 1], 0), x);
            const int nu = (opt.coarsening == LINA_AGGRESSIVE && l == f) ? opt.aggr_smoothing_iterations
                                                                          : opt.smoothing_iterations;
            smooth_warm<TX>(L, nu, b, x);
            run_rest<TX>(l, L, nu, b, x, false);
        }
        go(convert_kernel<TX, double>, gf, stream, lv[f].n, (const TX*)lvx<TX>(lv[f], 0), X);
    }

    // z = M^-1 r on the finest level (r FP64 on the device); mixed precision
    // leaves the result in kz32 (FP32), FP64 in z.
    void precondition(const double* r, double* z, bool time_it, bool apply_signs = true) {
        const int l = depth - 1;
        DLevel& L = lv[l];
        if (depth == 1) {
            if (opt.precision == LINA_PREC_MIXED) {
                go(convert_kernel<double, float>, grid_for(L.n, kThreads), stream, L.n, r, L.b32);
                coarse_solve<float>(L.b32, kz32);
            } else {
                coarse_solve<double>(r, z);
            }
            return;
        }
        const int nu = (opt.coarsening == LINA_AGGRESSIVE) ? opt.aggr_smoothing_iterations : opt.smoothing_iterations;
        const double* sign = (has_signs && apply_signs) ? signs : nullptr;
        if (opt.precision == LINA_PREC_MIXED) {
            presmooth<double, float>(L, nu, r, sign, isoinv, L.b32, kz32, time_it && l == timed_level);
            run_rest<float>(l, L, nu, L.b32, kz32, time_it);
        } else {
            double* b = const_cast<double*>(r);
            if (sign) b = L.b64;
            presmooth<double, double>(L, nu, r, sign, isoinv, b, z, time_it && l == timed_level);
            run_rest<double>(l, L, nu, b, z, time_it);
        }
    }

    const DCsr& krylov_matrix() const { return has_signs ? Aorig : lv[depth - 1].A; }

    // one PCG iteration: z = M^-1 r (unless reused), s = r.z, p = z + beta p, q = A p, x/r update
    // flexible beta (Polak-Ribiere form) by default for the mixed-precision preconditioner, whose FP32
    // rounding makes it vary slightly from one application to the next; the reference's beta = s/s_old
    // (PCGS.c:200) for FP64; LINA_PCG_BETA_* flags choose either explicitly
    int beta_mode = -1;
    int flexible_beta() const {
        if (beta_mode >= 0) return beta_mode;
        return opt.precision == LINA_PREC_MIXED ? 1 : 0;
    }
    // directions kept by the Krylov loop: FCG(m) for m >= 2 (mixed precision by default, where the FP32
    // V-cycle's rounding makes the preconditioner vary), 1 for the two-term recurrences above
    int history() const {
        if (beta_mode >= 0) return 1;  // an explicitly chosen two-term recurrence
        if (fcg_m > 0) return fcg_m;
        return opt.precision == LINA_PREC_MIXED ? kFcgDefault : 1;
    }
    static constexpr int kFcgDefault = 6;
    // the rings of kept directions (allocated before any capture)
    int ensure_history() {
        const int m = history();
        if (m < 2 || hist_m >= m) return 0;
        const size_t n = (size_t)lv[depth - 1].n;
        int rc;
        if ((rc = alloc(&kph, (size_t)m * n))) return rc;
        if ((rc = alloc(&kqh, (size_t)m * n))) return rc;
        hist_m = m;
        return 0;
    }
    template <int M>
    void issue_fcg_dots(int n, bool mixed, int gr) {
        if (mixed)
            go(fcg_dot_kernel<float, M>, gr, stream, n, (const double*)kr, (const float*)kz32, (const double*)kqh,
               partials, ticket, sc);
        else
            go(fcg_dot_kernel<double, M>, gr, stream, n, (const double*)kr, (const double*)kz, (const double*)kqh,
               partials, ticket, sc);
    }
    template <int M>
    void issue_fcg_p(int n, bool mixed, int gv) {
        if (mixed)
            go(fcg_update_p_kernel<float, M>, gv, stream, n, (const float*)kz32, (const double*)kph, kp,
               (const KScalars*)sc);
        else
            go(fcg_update_p_kernel<double, M>, gv, stream, n, (const double*)kz, (const double*)kph, kp,
               (const KScalars*)sc);
    }
    void issue_iteration(int n, bool precon, bool time_it) {
        const bool mixed = (opt.precision == LINA_PREC_MIXED);
        const int flexible = flexible_beta();
        const int gr = grid_red(n), gv = grid_for(n, kThreads);
        if (precon) precondition(kr, kz, time_it);
        const int m = history();
        if (m >= 2 && hist_m >= m) {
            switch (m) {
#define LINA_FCG_CASE(MM)              \
    case MM:                           \
        issue_fcg_dots<MM>(n, mixed, gr); \
        issue_fcg_p<MM>(n, mixed, gv);  \
        break;
                LINA_FCG_CASE(2)
                LINA_FCG_CASE(3)
                LINA_FCG_CASE(4)
                LINA_FCG_CASE(5)
                LINA_FCG_CASE(6)
                LINA_FCG_CASE(7)
                default:
                    LINA_FCG_CASE(8)
#undef LINA_FCG_CASE
            }
            csr<double, M_DOT>(krylov_matrix(), kp, kq);
            go(update_xr_kernel, gr, stream, n, kx, kr, (const double*)kp, (const double*)kq, partials, ticket, sc,
               m, kph, kqh);
            return;
        }
        if (mixed)
            go(dot_rz_kernel<float>, gr, stream, n, (const double*)kr, (const float*)kz32, (const double*)kq, flexible,
               partials, ticket, sc);
        else
            go(dot_rz_kernel<double>, gr, stream, n, (const double*)kr, (const double*)kz, (const double*)kq,
               flexible, partials, ticket, sc);
        if (mixed)
            go(update_p_kernel<float>, gv, stream, n, (const float*)kz32, kp, flexible, sc);
        else
            go(update_p_kernel<double>, gv, stream, n, (const double*)kz, kp, flexible, sc);
        csr<double, M_DOT>(krylov_matrix(), kp, kq);
        go(update_xr_kernel, gr, stream, n, kx, kr, (const double*)kp, (const double*)kq, partials, ticket, sc, 0,
           (double*)nullptr, (double*)nullptr);
    }

    // capture issue_iteration + the loop test into a while-loop graph (cached per configuration)
    int ensure_graph(int n) {
        if (gexec && g_prec == opt.precision && g_smoother == opt.smoother && g_omega == opt.omega &&
            g_flexible == flexible_beta() && g_history == history())
            return 0;
        drop_graph();
        cudaGraph_t g = nullptr;
        CK(cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle hd;
        cudaError_t e = cudaGraphConditionalHandleCreate(&hd, g, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams cp = {};
        cudaGraphNode_t node;
        if (e == cudaSuccess) {
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = hd;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
        }
        if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(stream, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                               cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            set_err("graph construction failed: %s", cudaGetErrorString(e));
            return LINA_GPU_ECUDA;
        }
        const unsigned long long before = g_launches;
        issue_iteration(n, true, false);
        loop_cond_kernel<<<1, 1, 0, stream>>>(hd, sc);
        g_kernels = (long)(g_launches - before) + 1;
        g_launches = before;
        cudaGraph_t body = nullptr;
        e = cudaStreamEndCapture(stream, &body);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            gexec = nullptr;
            set_err("graph capture/instantiation failed: %s", cudaGetErrorString(e));
            return LINA_GPU_ECUDA;
        }
        g_prec = opt.precision;
        g_smoother = opt.smoother;
        g_omega = opt.omega;
        g_flexible = flexible_beta();
        g_history = history();
        return 0;
    }
};

namespace {

// 64-bit fingerprint of a CSR pattern (row pointers and column indices): FNV-1a over fixed chunks, the
// chunk values combined in order
uint64_t pattern_fingerprint_csr(const lina::Csr& A) {
    const long np = (long)A.ptr.size(), nc = (long)A.col.size();
    constexpr long kChunk = 1L << 20;
    const long chunks = (np + kChunk - 1) / kChunk + (nc + kChunk - 1) / kChunk;
    std::vector<uint64_t> part(chunks);
#pragma omp parallel for schedule(static)
    for (long c = 0; c < chunks; c++) {
        const long pc = (np + kChunk - 1) / kChunk;
        const int* a = c < pc ? A.ptr.data() : A.col.data();
        const long n = c < pc ? np : nc;
        const long lo = (c < pc ? c : c - pc) * kChunk, hi = std::min(n, lo + kChunk);
        uint64_t h = 1469598103934665603ull;
        for (long k = lo; k < hi; k++) {
            h ^= (uint32_t)a[k];
            h *= 1099511628211ull;
        }
        part[c] = h;
    }
    uint64_t h = 1469598103934665603ull ^ (uint64_t)np ^ ((uint64_t)nc << 32);
    for (uint64_t v : part) {
        h ^= v;
        h *= 1099511628211ull;
    }
    return h;
}

// the Jacobi diagonal of a level (1/a_ii; 0 for a zero diagonal and for undecided rows of levels >= 1)
void level_dinv(const lina::HostLevel& hl, int l, std::vector<double>& dinv) {
    const int n = hl.A.n;
    dinv.assign(n, 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        double d = 0.0;
        for (int p = hl.A.ptr[i]; p < hl.A.ptr[i + 1]; p++)
            if (hl.A.col[p] == i) d = hl.A.val[p];
        const bool skip = (l > 0 && !hl.labels.empty() && hl.labels[i] == lina::kUndecided);
        dinv[i] = (skip || d == 0.0) ? 0.0 : 1.0 / d;
    }
}

// The groups of a segmented level for the cluster-fused multicolour-SOR step: consecutive whole systems
// while their rows fit g_fused_rows.  Built only where every row of a group couples only to rows of its
// group (A), every restricted row reads only its rows (R), and every prolongated row only its coarse rows
// (P): then each cluster's reads and stores of its copy of x stay inside the copy.
int build_fused_groups(lina_gpu_amg* h, int l, const lina::HostLevel& hl,
                       const std::vector<std::vector<int>>& colours) {
    DLevel& L = h->lv[l];
    const std::vector<int>& off = h->seg_off[l];
    const std::vector<int>& coff = h->seg_off[l - 1];
    const int S = (int)off.size() - 1;
    if (!g_fused_groups || g_fused_rows <= 0 || L.Acol.lanes <= 0 || L.A.lanes <= 0 || L.R.lanes <= 0 ||
        L.P.lanes <= 0 || L.n <= g_fused_rows || L.ncolours <= 0)
        return 0;
    std::vector<int4> grp;  // (r0, r1, c0, c1)
    for (int i = 0; i < S;) {
        if (off[i + 1] - off[i] > g_fused_rows) return 0;  // a system too large for one cluster
        int j = i + 1;
        while (j < S && off[j + 1] - off[i] <= g_fused_rows) j++;
        grp.push_back(make_int4(off[i], off[j], coff[i], coff[j]));
        i = j;
    }
    auto inside = [](const lina::Csr& M, int row0, int row1, int col0, int col1) {
        for (int r = row0; r < row1; r++)
            for (int p = M.ptr[r]; p < M.ptr[r + 1]; p++)
                if (M.col[p] < col0 || M.col[p] >= col1) return false;
        return true;
    };
    for (const int4& g : grp)
        if (!inside(hl.A, g.x, g.y, g.x, g.y) || !inside(hl.R, g.z, g.w, g.x, g.y) || !inside(hl.P, g.x, g.y, g.z, g.w))
            return 0;
    // per group and colour: the positions of the group's rows of that colour in the colour order
    const int G = (int)grp.size(), C = L.ncolours;
    std::vector<int2> ranges((size_t)G * C);
    for (int c = 0; c < C; c++) {
        const std::vector<int>& rows = colours[c];
        const int base = L.Acol.group_row[c];
        for (int k = 0; k < G; k++) {
            const int b0 = (int)(std::lower_bound(rows.begin(), rows.end(), grp[k].x) - rows.begin());
            const int b1 = (int)(std::lower_bound(rows.begin(), rows.end(), grp[k].y) - rows.begin());
            ranges[(size_t)k * C + c] = make_int2(base + b0, base + b1);
        }
    }
    int2* d_ranges = nullptr;
    int rc;
    if ((rc = h->upload(&d_ranges, ranges.data(), ranges.size()))) return rc;
    std::vector<FusedGroup> fg(G);
    int most = 0;
    for (int k = 0; k < G; k++) {
        fg[k] = FusedGroup{grp[k].x, grp[k].y, grp[k].z, grp[k].w, d_ranges + (size_t)k * C};
        most = std::max(most, grp[k].y - grp[k].x);
    }
    if ((rc = h->upload(&L.d_groups, fg.data(), fg.size()))) return rc;
    CK(cudaStreamSynchronize(h->stream));
    L.ngroups = G;
    L.max_group_rows = most;
    return 0;
}

// Layout autotuning of one level: the level's matrix uploaded in each candidate layout (one thread per
// row, i.e. SELL-32 and for FP32 the quad layout; or 4, 8 or 16 lanes per row), timed with CUDA events
// over 5 smoother sweeps plus a residual in the hierarchy's precision (multicolour SOR: every colour of
// a sweep), after 2 untimed sweeps.  The rule's layout is kept unless another is at least 5 % faster
// (FP32 natural-order passes of levels of 20,000 rows or more read the quad layout whatever the lane
// count, so there the candidates differ by noise).  The temporary uploads are released.
template <typename TX>
int autotune_level(lina_gpu_amg* h, const lina::HostLevel& hl, int l, const std::vector<std::vector<int>>& colours,
                   int* best_out) {
    const int n = hl.A.n;
    const bool sor = h->opt.smoother == LINA_SMOOTHER_MC_SOR;
    const size_t mark = h->allocations.size();
    const long mark_bytes = h->dev_bytes;
    int rc = 0;
    TX *x = nullptr, *y = nullptr, *b = nullptr, *dv = nullptr;
    std::vector<double> d64;
    level_dinv(hl, l, d64);
    std::vector<TX> dinv(d64.begin(), d64.end()), ones(n, TX(1));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float best_ms = 0.f;
    int best = -1;
    const TX w = TX(h->opt.omega);
    std::string report;
    const int rule = h->lanes_rows > 0 ? csrv_lanes_for_shape(std::min<long>(h->lanes_rows, n),
                                                               n > 0 ? double(hl.A.nnz()) / n : 0.0)
                                        : csrv_lanes_for(hl.A);
    float rule_ms = 0.f;
    if ((rc = h->alloc(&x, n)) || (rc = h->alloc(&y, n)) || (rc = h->upload(&b, ones.data(), ones.size())) ||
        (rc = h->upload(&dv, dinv.data(), dinv.size())))
        goto done;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = LINA_GPU_ECUDA;
        goto done;
    }
    for (int cand : {0, 4, 8, 16}) {
        DCsr A, Ac;
        h->force_lanes = cand;
        rc = h->upload_csr(A, hl.A);
        if (!rc && sor) rc = h->upload_csr(Ac, hl.A, &colours);
        h->force_lanes = -1;
        if (rc) goto done;
        CK(cudaMemsetAsync(x, 0, (size_t)n * sizeof(TX), h->stream));
        auto sweep = [&]() {
            if (sor) {
                for (int c = 0; c < (int)colours.size(); c++) h->csr_group<TX, M_SOR>(Ac, c, x, x, b, dv, w);
            } else {
                h->csr<TX, M_JACOBI>(A, x, y, b, dv, w);
                std::swap(x, y);
            }
        };
        for (int k = 0; k < 2; k++) sweep();
        cudaEventRecord(e0, h->stream);
        for (int k = 0; k < 5; k++) sweep();
        h->csr<TX, M_RESID>(A, x, y, b);
        cudaEventRecord(e1, h->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            rc = LINA_GPU_ECUDA;
            goto done;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        char buf[64];
        snprintf(buf, sizeof buf, " %s %.1f us", cand ? (std::to_string(cand) + " lanes").c_str() : "one thread",
                 ms * 1e3 / 5);
        report += buf;
        if (cand == rule) rule_ms = ms;
        if (best < 0 || ms < best_ms) {
            best_ms = ms;
            best = cand;
        }
    }
    if (rule_ms > 0.f && best_ms > 0.95f * rule_ms) best = rule;
    if (getenv("LINA_SETUP_TIMING"))
        fprintf(stderr, "autotune level %d (%d rows, %ld entries):%s per sweep -> %s\n", l, n, (long)hl.A.nnz(),
                report.c_str(), best ? (std::to_string(best) + " lanes").c_str() : "one thread");
done:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(h->stream);
    for (size_t k = mark; k < h->allocations.size(); k++) cudaFree(h->allocations[k]);
    h->allocations.resize(mark);
    h->dev_bytes = mark_bytes;
    if (!rc) *best_out = best;
    return rc;
}

// the value images of a staged level, from its current entries and 1/a_ii
int stage_refresh(lina_gpu_amg* h, DLevel& L) {
    if (L.stage_k <= 0) return 0;
    const long n = (long)L.stage_k * L.stage_nvals;
    go(stage_gather_kernel, grid_for(n, kThreads), h->stream, n, (const int*)L.stage_src, (const double*)L.Acol.v64,
       (const float*)L.Acol.v32, (const double*)L.dinv64, (const float*)L.dinv32, h->opt.omega, L.stage_v64,
       L.stage_v32);
    CK(cudaGetLastError());
    return 0;
}

static inline int pad4(long v) { return (int)((v + 3) / 4 * 4); }

// The staged plan of a level (see staged_step_kernel) for a cluster of K blocks, the largest the GPU
// schedules (16 on GB300; LINA_STAGED_K=1|2|4|8 asks for fewer); none where the images, with a copy of
// x, do not fit a block's shared memory in FP64 (such levels' fused steps read the matrix from global
// memory).  The largest cluster is the fastest: GB300's SM runs one FP64 warp instruction about every
// 19 cycles, whatever its active lanes, so a colour of many rows is bound by the FP64 pipes of the
// blocks that share it (P1 Poisson 257 x 257, FP64 solves: 10.3 ms with one block per level, 9.6 with
// four, 8.7 with eight, 8.6 with sixteen).
int build_stage(lina_gpu_amg* h, DLevel& L, const lina::Csr& A, const std::vector<std::vector<int>>& groups) {
    L.stage_k = 0;
    const int n = L.n, C = L.ncolours, S = L.Acol.lanes;
    if (S <= 0 || C <= 0 || (long)n * 8 > kStagedSmemMax || (int)groups.size() != C) return 0;
    // every variant's launch attributes are set here, outside any stream capture
    int K = std::min(std::min(lina_gpu_amg::staged_cluster_max<double, true>(),
                              lina_gpu_amg::staged_cluster_max<double, false>()),
                     std::min(lina_gpu_amg::staged_cluster_max<float, true>(),
                              lina_gpu_amg::staged_cluster_max<float, false>()));
    if (const char* e = getenv("LINA_STAGED_K")) {
        const int v = atoi(e);
        if (v == 1 || v == 2 || v == 4 || v == 8 || v == 16) K = std::min(K, v);
    }
    auto share = [&](int c, int r, int& a, int& b) {
        const long len = (long)groups[c].size();
        a = (int)(len * r / K);
        b = (int)(len * (r + 1) / K);
    };
    int pmax = 0;
    long emax = 0;
    for (int r = 0; r < K; r++) {
        int P = 0;
        long E = 0;
        for (int c = 0; c < C; c++) {
            int a, b;
            share(c, r, a, b);
            P += b - a;
            for (int t = a; t < b; t++) E += A.ptr[groups[c][t] + 1] - A.ptr[groups[c][t]];
        }
        pmax = std::max(pmax, P);
        emax = std::max(emax, E);
    }
    const int o_row = pad4(C + 1), o_off = o_row + pad4(pmax), o_col = o_off + pad4(pmax + 1);
    const long ints = (long)o_col + pad4(emax);
    const long nvals = (long)pad4(emax) + pad4(pmax);
    const long bytes = ((long)n * 8 + 15) / 16 * 16 + (nvals + pad4(pmax)) * 8 + ints * 4;
    if (bytes > kStagedSmemMax) return 0;
    std::vector<int> img((size_t)K * ints, 0), src((size_t)K * nvals, -1);
    for (int r = 0; r < K; r++) {
        int* I = img.data() + (size_t)r * ints;
        int* V = src.data() + (size_t)r * nvals;
        int q = 0, e = 0;
        for (int c = 0; c < C; c++) {
            I[c] = q;
            int a, b;
            share(c, r, a, b);
            for (int t = a; t < b; t++, q++) {
                const int i = groups[c][t];
                I[o_row + q] = i;
                I[o_off + q] = e;
                V[pad4(emax) + q] = -2 - i;
                for (int k = A.ptr[i]; k < A.ptr[i + 1]; k++, e++) {
                    I[o_col + e] = (A.col[k] >= 0 && A.col[k] < n) ? A.col[k] : 0;  // placeholders hold 0.0
                    V[e] = k;
                }
            }
        }
        I[C] = q;
        I[o_off + q] = e;
    }
    int rc;
    if ((rc = h->upload(&L.stage_int, img.data(), img.size()))) return rc;
    if ((rc = h->upload(&L.stage_src, src.data(), src.size()))) return rc;
    if ((rc = h->alloc(&L.stage_v64, src.size()))) return rc;
    if ((rc = h->alloc(&L.stage_v32, src.size()))) return rc;
    L.stage_k = K;
    L.stage_ints = (int)ints;
    L.stage_nvals = (int)nvals;
    L.stage_pslots = pad4(pmax);
    L.stage_o_row = o_row;
    L.stage_o_off = o_off;
    L.stage_o_col = o_col;
    L.stage_o_dinv = pad4(emax);
    if ((rc = stage_refresh(h, L))) return rc;
    // the host images must outlive the asynchronous uploads
    return cudaStreamSynchronize(h->stream) == cudaSuccess ? 0 : LINA_GPU_ECUDA;
}

int upload_hierarchy(lina_gpu_amg* h) {
    lina::HostHierarchy& H = h->host;
    const int depth = h->depth;
    h->lv.assign(depth, DLevel());
    int rc;
    for (int l = 0; l < depth; l++) {
        lina::HostLevel& hl = H.lv[l];
        DLevel& L = h->lv[l];
        L.n = hl.A.n;
        h->lanes_rows = h->seg_max_rows.empty() ? 0 : h->seg_max_rows[l];
        // layout autotuning of the levels below the finest (their choice is kept for re-uploads)
        // (levels of more than 50M entries, and the finest level, keep the rule: one thread per row, and
        // their candidate uploads would cost seconds.  Measured on the 96-system segmented batch: its
        // levels of 100M and 153M entries time fastest with one thread per row, as the rule chooses, and
        // tuning them doubled the batch's creation time, 9 s to 18 s)
        if (h->autotune && l > 0 && l < depth - 1 && hl.A.n >= 2000 && hl.A.nnz() <= 50000000L) {
            if ((int)h->tuned_lanes.size() != depth) h->tuned_lanes.assign(depth, -1);
            if (h->tuned_lanes[l] < 0) {
                std::vector<int> colour;
                std::vector<std::vector<int>> cgroups;
                if (h->opt.smoother == LINA_SMOOTHER_MC_SOR) {
                    const int nc = lina::greedy_colouring(hl.A, colour);
                    cgroups.assign(nc, std::vector<int>());
                    for (int i = 0; i < L.n; i++) cgroups[colour[i]].push_back(i);
                }
                int best = -1;
                rc = h->opt.precision == LINA_PREC_MIXED ? autotune_level<float>(h, hl, l, cgroups, &best)
                                                         : autotune_level<double>(h, hl, l, cgroups, &best);
                if (rc) return rc;
                h->tuned_lanes[l] = best;
            }
        }
        h->force_lanes = ((int)h->tuned_lanes.size() == depth) ? h->tuned_lanes[l] : -1;
        std::vector<int> posA, posQ, posC;
        if ((rc = h->upload_csr(L.A, hl.A, nullptr, h->keep_maps ? &posA : nullptr, h->keep_maps ? &posQ : nullptr)))
            return rc;
        std::vector<double> dinv;
        level_dinv(hl, l, dinv);
        std::vector<float> dinv32(dinv.begin(), dinv.end());
        if ((rc = h->upload(&L.dinv64, dinv.data(), dinv.size()))) return rc;
        if ((rc = h->upload(&L.dinv32, dinv32.data(), dinv32.size()))) return rc;
        if (l > 0) {
            const int tuned = h->force_lanes;  // the autotuned layout is A's (and its colour-grouped copy's)
            h->force_lanes = -1;
            if ((rc = h->upload_csr(L.P, hl.P))) return rc;
            if ((rc = h->upload_csr(L.R, hl.R))) return rc;
            h->force_lanes = tuned;
            std::vector<int> colour;
            L.ncolours = lina::greedy_colouring(hl.A, colour);
            std::vector<std::vector<int>> groups(L.ncolours);
            for (int i = 0; i < L.n; i++) groups[colour[i]].push_back(i);
            if ((rc = h->upload_csr(L.Acol, hl.A, &groups, h->keep_maps ? &posC : nullptr))) return rc;
            if ((rc = build_stage(h, L, hl.A, groups))) return rc;
            if (!h->seg_off.empty() && (rc = build_fused_groups(h, l, hl, groups))) return rc;
        }
        if (h->keep_maps) {  // in-place value updates of later recomputes
            if ((int)h->rmaps.size() != depth) h->rmaps.assign(depth, lina_gpu_amg::LevelMaps());
            lina_gpu_amg::LevelMaps& M = h->rmaps[l];
            const long nnz = hl.A.nnz();
            auto up = [&](int** dst, std::vector<int>& pos) -> int {
                if (pos.empty()) {  // values in CSR order (lane-group layout)
                    pos.resize(nnz);
                    for (long k = 0; k < nnz; k++) pos[k] = (int)k;
                }
                return h->upload(dst, pos.data(), pos.size());
            };
            if ((rc = up(&M.posA, posA))) return rc;
            M.posQ = nullptr;
            if (L.A.q_val && !posQ.empty() && (rc = h->upload(&M.posQ, posQ.data(), posQ.size()))) return rc;
            M.posC = nullptr;
            if (l > 0 && (rc = up(&M.posC, posC))) return rc;
            M.pattern = pattern_fingerprint_csr(hl.A);
            M.nnz = nnz;
            CK(cudaStreamSynchronize(h->stream));  // the host maps go out of scope
        }
        h->force_lanes = -1;
        // work vectors
        if ((rc = h->alloc(&L.x64, L.n))) return rc;
        if ((rc = h->alloc(&L.t64, L.n))) return rc;
        if ((rc = h->alloc(&L.b64, L.n))) return rc;
        if ((rc = h->alloc(&L.r64, L.n))) return rc;
        if ((rc = h->alloc(&L.x32, L.n))) return rc;
        if ((rc = h->alloc(&L.t32, L.n))) return rc;
        if ((rc = h->alloc(&L.b32, L.n))) return rc;
        if ((rc = h->alloc(&L.r32, L.n))) return rc;
    }
    h->lanes_rows = 0;
    // coarsest block
    lina::CoarseSolver& cs = H.coarse;
    h->cm = (int)cs.block_rows.size();
    h->c_block_rows = cs.block_rows;
    std::vector<int> blockpos(cs.n, 0);
    for (int k = 0; k < h->cm; k++) blockpos[cs.block_rows[k]] = k;
    if ((rc = h->upload(&h->c_brows, cs.block_rows.data(), cs.block_rows.size()))) return rc;
    if ((rc = h->upload(&h->c_inblock, cs.in_block.data(), cs.in_block.size()))) return rc;
    if ((rc = h->upload(&h->c_blockpos, blockpos.data(), blockpos.size()))) return rc;
    if ((rc = h->upload(&h->c_inv, cs.inv.data(), cs.inv.size()))) return rc;
    if (cs.blocks.empty()) {
        if (!cs.inverted) {  // a large block: inverted in place on the device
            int* err = nullptr;
            if ((rc = h->alloc(&err, 1))) return rc;
            std::string msg;
            if ((rc = lina::dense_inverse(h->cm, h->c_inv, g_dense_method, h->stream, err, msg))) {
                set_err("%s", msg.c_str());
                return rc;
            }
        }
    } else {  // block-diagonal: each block's inverse at its offset, large ones inverted on the device
        const int nb = (int)cs.blocks.size() - 1;
        std::vector<int> rblk(std::max(h->cm, 1), 0);
        for (int k = 0; k < nb; k++)
            for (int r = cs.blocks[k]; r < cs.blocks[k + 1]; r++) rblk[r] = k;
        if ((rc = h->upload(&h->c_rblk, rblk.data(), rblk.size()))) return rc;
        if ((rc = h->upload(&h->c_boff, cs.blocks.data(), cs.blocks.size()))) return rc;
        if ((rc = h->upload(&h->c_ioff, cs.inv_offsets.data(), cs.inv_offsets.size()))) return rc;
        int* err = nullptr;
        for (int k = 0; k < nb; k++) {
            if (cs.block_inverted[k]) continue;
            if (!err && (rc = h->alloc(&err, 1))) return rc;
            std::string msg;
            if ((rc = lina::dense_inverse(cs.blocks[k + 1] - cs.blocks[k], h->c_inv + cs.inv_offsets[k],
                                          g_dense_method, h->stream, err, msg))) {
                set_err("%s", msg.c_str());
                return rc;
            }
        }
    }
    if ((rc = h->upload(&h->c_dginv, cs.diag_inv.data(), cs.diag_inv.size()))) return rc;
    if ((rc = h->alloc(&h->c_bblk, std::max(h->cm, 1)))) return rc;
    // finest extras
    const int nf = H.lv[depth - 1].A.n;
    {
        std::vector<double> iso(nf, 0.0);
        if (depth > 1) {
            const lina::HostLevel& F = H.lv[depth - 1];
            for (int i = 0; i < nf; i++)
                if (F.labels[i] == lina::kIsolated)
                    for (int p = F.A.ptr[i]; p < F.A.ptr[i + 1]; p++)
                        if (F.A.val[p] != 0.0) {
                            iso[i] = 1.0 / F.A.val[p];
                            break;
                        }
        }
        if ((rc = h->upload(&h->isoinv, iso.data(), iso.size()))) return rc;
    }
    h->has_signs = false;
    for (double s : H.signs)
        if (s < 0) h->has_signs = true;
    if (h->has_signs) {
        if ((rc = h->upload(&h->signs, H.signs.data(), H.signs.size()))) return rc;
    }
    if ((rc = h->alloc(&h->kr, nf))) return rc;
    if ((rc = h->alloc(&h->kz, nf))) return rc;
    if ((rc = h->alloc(&h->kp, nf))) return rc;
    if ((rc = h->alloc(&h->kq, nf))) return rc;
    if ((rc = h->alloc(&h->kx, nf))) return rc;
    if ((rc = h->alloc(&h->kb, nf))) return rc;
    if ((rc = h->alloc(&h->kt, nf))) return rc;
    if ((rc = h->alloc(&h->kz32, nf))) return rc;
    if ((rc = h->alloc(&h->partials, (kFcgMax + 1) * kMaxBlocks))) return rc;
    if ((rc = h->alloc(&h->ticket, 4))) return rc;
    if ((rc = h->alloc(&h->sc, 1))) return rc;
    if ((rc = h->alloc(&h->hscal, 2))) return rc;
    CK(cudaMemsetAsync(h->ticket, 0, 4 * sizeof(unsigned), h->stream));
    CK(cudaMemsetAsync(h->sc, 0, sizeof(KScalars), h->stream));
    if (!h->sc_host) CK(cudaMallocHost((void**)&h->sc_host, sizeof(KScalars)));
    CK(cudaStreamSynchronize(h->stream));
    h->timed_level = depth - 1;
    for (int l = 1; l < depth; l++)
        if (h->lv[l].A.nnz > h->lv[h->timed_level].A.nnz) h->timed_level = l;
    return 0;
}

lina::Csr csr_from(int n, const int* rowptr, const int* col, const double* val) {
    lina::Csr A;
    A.n = n;
    A.ncols = n;
    A.ptr.assign(rowptr, rowptr + n + 1);
    long nnz = rowptr[n];
    A.col.assign(col, col + nnz);
    A.val.assign(val, val + nnz);
    return A;
}

bool valid_csr(int n, const int* rowptr, const int* col) {
    if (n <= 0 || !rowptr || !col || rowptr[0] != 0) return false;
    for (int i = 0; i < n; i++) {
        if (rowptr[i + 1] < rowptr[i]) return false;
        for (int p = rowptr[i]; p < rowptr[i + 1]; p++) {
            if (col[p] < 0 || col[p] >= n) return false;
            if (p > rowptr[i] && col[p] <= col[p - 1]) return false;
        }
    }
    return true;
}

// true residual b - A x (FP64), norm into sc->norm2; result left in kt
int true_residual(lina_gpu_amg* h, const double* b, const double* x) {
    const DCsr& A = h->krylov_matrix();
    h->csr<double, M_RESID>(A, x, h->kt, b);
    go(norm2_kernel<double>, grid_red(A.n), h->stream, A.n, h->kt, h->partials, h->ticket, h->sc);
    return 0;
}

int read_scalars(lina_gpu_amg* h) {
    CK(cudaMemcpyAsync(h->sc_host, h->sc, sizeof(KScalars), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

}  // namespace

namespace lina {
namespace dev {
void set_error(const char* msg) { g_err = msg ? msg : ""; }
}  // namespace dev
}  // namespace lina

// =================================================================== C-ABI
extern "C" {

void lina_gpu_default_options(lina_gpu_amg_options* o) {
    if (!o) return;
    o->dof = 1;
    o->depth = 2;
    o->smoothing_iterations = 2;
    o->aggr_smoothing_iterations = 2;
    o->coarsening = LINA_STANDARD;
    o->eps_minus = 0.3;
    o->eps_plus = 0.5;
    o->matrix_tol = 0.1;
    o->smoother = LINA_SMOOTHER_JACOBI;
    o->omega = 0.6;
    o->precision = LINA_PREC_FP64;
}

const char* lina_gpu_last_error(void) { return g_err.c_str(); }

int lina_gpu_set_fused_rows(int max_rows) {
    if (max_rows < 0) {
        set_err("lina_gpu_set_fused_rows: max_rows must be >= 0");
        return LINA_GPU_EINVAL;
    }
    g_fused_rows = max_rows;
    return 0;
}

int lina_gpu_set_autotune(int on) {
    g_autotune = on ? 1 : 0;
    return 0;
}

int lina_gpu_set_fused_groups(int on) {
    g_fused_groups = on ? 1 : 0;
    return 0;
}

int lina_gpu_set_fused_jacobi_entries(long max_entries) {
    if (max_entries < 0) {
        set_err("lina_gpu_set_fused_jacobi_entries: max_entries must be >= 0");
        return LINA_GPU_EINVAL;
    }
    g_fused_jacobi_entries = max_entries;
    return 0;
}

int lina_gpu_set_layout(int layout) {
    if (layout < 0 || layout > 6) {
        set_err("lina_gpu_set_layout: layout must be 0 to 6");
        return LINA_GPU_EINVAL;
    }
    g_layout = layout;
    return 0;
}

int lina_gpu_set_coarse_inverse(int min_rows, int method) {
    if (min_rows < 0 || (method != LINA_DENSE_SIMT && method != LINA_DENSE_DMMA)) {
        set_err("lina_gpu_set_coarse_inverse: invalid argument");
        return LINA_GPU_EINVAL;
    }
    g_coarse_device_rows = min_rows;
    g_dense_method = method;
    return 0;
}

int lina_gpu_set_device_memory_limit(long bytes) {
    if (bytes < 0) {
        set_err("lina_gpu_set_device_memory_limit: negative limit");
        return LINA_GPU_EINVAL;
    }
    g_mem_limit = bytes;
    return 0;
}

int lina_gpu_set_pdl(int on) {
    g_pdl = on ? 1 : 0;
    return 0;
}

int lina_gpu_set_sell_quads(int on) {
    g_quads = on ? 1 : 0;
    return 0;
}

int lina_gpu_set_sell_index_bits(int bits) {
    if (bits != 16 && bits != 32) {
        set_err("lina_gpu_set_sell_index_bits: bits must be 16 or 32");
        return LINA_GPU_EINVAL;
    }
    g_sell_bits = bits;
    return 0;
}

int lina_gpu_set_device(int device) {
    CK(cudaSetDevice(device));
    return 0;
}

int lina_gpu_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

static int amg_create_impl(int n, const int* rowptr, const int* col, const double* val,
                           const lina_gpu_amg_options* opt, lina_gpu_amg** out, bool host_only) {
    if (!out || !opt || !val || !valid_csr(n, rowptr, col)) {
        set_err("lina_gpu_amg_create: invalid CSR input or options");
        return LINA_GPU_EINVAL;
    }
    if (opt->depth < 1 || opt->dof < 1 || opt->smoothing_iterations < 0 || opt->aggr_smoothing_iterations < 0 ||
        (opt->smoother != LINA_SMOOTHER_JACOBI && opt->smoother != LINA_SMOOTHER_MC_SOR) ||
        (opt->precision != LINA_PREC_FP64 && opt->precision != LINA_PREC_MIXED)) {
        set_err("lina_gpu_amg_create: invalid options");
        return LINA_GPU_EINVAL;
    }
    *out = nullptr;
    lina_gpu_amg* h = new lina_gpu_amg();
    h->autotune = g_autotune != 0;
    h->opt = *opt;
    h->depth = opt->depth;
    lina::AmgParams p;
    p.dof = opt->dof;
    p.depth = opt->depth;
    p.smoothing_iterations = opt->smoothing_iterations;
    p.aggr_smoothing_iterations = opt->aggr_smoothing_iterations;
    p.coarsening = opt->coarsening == LINA_AGGRESSIVE ? lina::kAggressive
                   : opt->coarsening == LINA_PMIS     ? lina::kPmis
                                                      : lina::kStandard;
    p.eps_minus = opt->eps_minus;
    p.eps_plus = opt->eps_plus;
    p.matrix_tol = opt->matrix_tol;
    p.gpu_products = !host_only;  // the Galerkin products on the GPU (bit-identical to the host's)
    p.coarse_device_rows = host_only ? 0 : g_coarse_device_rows;
    if (!lina::amg_setup_host(csr_from(n, rowptr, col, val), p, h->host)) {
        set_err("AMG setup: %s", h->host.error.c_str());
        delete h;
        return LINA_GPU_ESETUP;
    }
    if (host_only) {
        h->host_only = true;
        *out = h;
        return 0;
    }
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_err("cudaStreamCreate failed");
        delete h;
        return LINA_GPU_ECUDA;
    }
    int rc = upload_hierarchy(h);
    if (rc) {
        delete h;
        return rc;
    }
    if (h->has_signs) {
        rc = h->upload_csr(h->Aorig, csr_from(n, rowptr, col, val));
        if (rc) {
            delete h;
            return rc;
        }
    }
    *out = h;
    return 0;
}

int lina_gpu_amg_create(int n, const int* rowptr, const int* col, const double* val,
                        const lina_gpu_amg_options* opt, lina_gpu_amg** out) {
    return amg_create_impl(n, rowptr, col, val, opt, out, false);
}

int lina_gpu_amg_create_host_only(int n, const int* rowptr, const int* col, const double* val,
                                  const lina_gpu_amg_options* opt, lina_gpu_amg** out) {
    return amg_create_impl(n, rowptr, col, val, opt, out, true);
}

int lina_gpu_amg_save(const lina_gpu_amg* h, const char* dir) {
    if (!h || !dir) {
        set_err("lina_gpu_amg_save: invalid argument");
        return LINA_GPU_EINVAL;
    }
    mkdir(dir, 0755);  // may exist already; a failure shows when the files are written
    std::string err;
    if (!lina::amg_save_host(h->host, dir, err)) {
        set_err("%s", err.c_str());
        return LINA_GPU_EINVAL;
    }
    return 0;
}

int lina_gpu_amg_load(const char* dir, const lina_gpu_amg_options* opt, int host_only, lina_gpu_amg** out) {
    if (!dir || !opt || !out ||
        (opt->smoother != LINA_SMOOTHER_JACOBI && opt->smoother != LINA_SMOOTHER_MC_SOR) ||
        (opt->precision != LINA_PREC_FP64 && opt->precision != LINA_PREC_MIXED) || opt->smoothing_iterations < 0 ||
        opt->aggr_smoothing_iterations < 0) {
        set_err("lina_gpu_amg_load: invalid argument");
        return LINA_GPU_EINVAL;
    }
    *out = nullptr;
    lina_gpu_amg* h = new lina_gpu_amg();
    h->autotune = g_autotune != 0;
    if (!lina::amg_load_host(dir, h->host, host_only ? 0 : g_coarse_device_rows)) {
        set_err("AMG load: %s", h->host.error.c_str());
        delete h;
        return LINA_GPU_EINVAL;
    }
    // the hierarchy's own structure; the caller's options for the solve phase
    const lina::AmgParams& p = h->host.params;
    h->opt = *opt;
    h->opt.depth = p.depth;
    h->opt.dof = p.dof;
    h->opt.coarsening = p.coarsening == lina::kAggressive ? LINA_AGGRESSIVE
                        : p.coarsening == lina::kPmis     ? LINA_PMIS
                                                          : LINA_STANDARD;
    h->opt.eps_minus = p.eps_minus;
    h->opt.eps_plus = p.eps_plus;
    h->opt.matrix_tol = p.matrix_tol;
    h->host.params.smoothing_iterations = opt->smoothing_iterations;
    h->host.params.aggr_smoothing_iterations = opt->aggr_smoothing_iterations;
    h->host.params.gpu_products = !host_only;
    h->depth = p.depth;
    if (host_only) {
        h->host_only = true;
        *out = h;
        return 0;
    }
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_err("cudaStreamCreate failed");
        delete h;
        return LINA_GPU_ECUDA;
    }
    int rc = upload_hierarchy(h);
    if (!rc && h->has_signs) {
        // the caller's matrix: the finest rows flipped back (the flip is an exact negation)
        lina::Csr A = h->host.lv[h->depth - 1].A;
        for (int i = 0; i < A.n; i++)
            if (h->host.signs[i] < 0)
                for (int q = A.ptr[i]; q < A.ptr[i + 1]; q++) A.val[q] = -A.val[q];
        rc = h->upload_csr(h->Aorig, A);
    }
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return 0;
}

}  // extern "C"

namespace {

// New values of every level on unchanged patterns (lina_gpu_amg_recompute after the first): each level's
// entries scattered into its device layouts, its Jacobi diagonal, the finest isolated-row inverses and
// the coarse inverse replaced in place; the device pointers (and a captured solve graph) stay valid.
// Returns 0, 1 when some pattern (or the coarse block) differs from the uploaded one, or an error.
int refresh_values(lina_gpu_amg* h) {
    const lina::HostHierarchy& H = h->host;
    const int depth = h->depth;
    if ((int)h->rmaps.size() != depth) return 1;
    for (int l = 0; l < depth; l++)
        if (H.lv[l].A.nnz() != h->rmaps[l].nnz || pattern_fingerprint_csr(H.lv[l].A) != h->rmaps[l].pattern) return 1;
    if (H.coarse.block_rows != h->c_block_rows || !H.coarse.blocks.empty()) return 1;
    long most = 0;
    for (int l = 0; l < depth; l++) most = std::max<long>(most, H.lv[l].A.nnz());
    int rc;
    if (most > h->rstage_n) {
        if ((rc = h->alloc(&h->rstage, most))) return rc;
        h->rstage_n = most;
    }
    cudaStream_t st = h->stream;
    for (int l = 0; l < depth; l++) {
        const lina::HostLevel& hl = H.lv[l];
        DLevel& L = h->lv[l];
        const lina_gpu_amg::LevelMaps& M = h->rmaps[l];
        CK(cudaMemcpyAsync(h->rstage, hl.A.val.data(), hl.A.nnz() * sizeof(double), cudaMemcpyHostToDevice, st));
        go(update_values_kernel, grid_for(hl.A.nnz(), kThreads), st, (long)hl.A.nnz(), (const double*)h->rstage,
           (const int*)M.posA, (const int*)M.posC, L.A.v64, L.A.v32, L.Acol.v64, L.Acol.v32, (const int*)M.posQ,
           reinterpret_cast<float*>(L.A.q_val));
        std::vector<double> dinv;
        level_dinv(hl, l, dinv);
        std::vector<float> dinv32(dinv.begin(), dinv.end());
        CK(cudaMemcpyAsync(L.dinv64, dinv.data(), dinv.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(L.dinv32, dinv32.data(), dinv32.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        if ((rc = stage_refresh(h, L))) return rc;
        CK(cudaStreamSynchronize(st));  // the staging buffer and the host vectors are reused
    }
    // coarsest level: the new dense block (inverted here or on the device) and 1/a_ii elsewhere
    const lina::CoarseSolver& cs = H.coarse;
    CK(cudaMemcpyAsync(h->c_inv, cs.inv.data(), cs.inv.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    if (!cs.inverted) {
        if (!h->rerr && (rc = h->alloc(&h->rerr, 1))) return rc;
        std::string msg;
        if ((rc = lina::dense_inverse(h->cm, h->c_inv, g_dense_method, st, h->rerr, msg))) {
            set_err("%s", msg.c_str());
            return rc;
        }
    }
    CK(cudaMemcpyAsync(h->c_dginv, cs.diag_inv.data(), cs.diag_inv.size() * sizeof(double), cudaMemcpyHostToDevice,
                       st));
    // the finest level's isolated rows
    const int nf = H.lv[depth - 1].A.n;
    std::vector<double> iso(nf, 0.0);
    if (depth > 1) {
        const lina::HostLevel& F = H.lv[depth - 1];
        for (int i = 0; i < nf; i++)
            if (F.labels[i] == lina::kIsolated)
                for (int p = F.A.ptr[i]; p < F.A.ptr[i + 1]; p++)
                    if (F.A.val[p] != 0.0) {
                        iso[i] = 1.0 / F.A.val[p];
                        break;
                    }
    }
    CK(cudaMemcpyAsync(h->isoinv, iso.data(), iso.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    // the finest-level update maps of lina_gpu_amg_update_values stay valid (same pattern and layouts)
    return 0;
}

}  // namespace

extern "C" {

int lina_gpu_amg_recompute(lina_gpu_amg* h, int n, const int* rowptr, const int* col, const double* val) {
    if (!h || !valid_csr(n, rowptr, col) || !val) {
        set_err("lina_gpu_amg_recompute: invalid input");
        return LINA_GPU_EINVAL;
    }
    if (!lina::amg_recompute_host(h->host, csr_from(n, rowptr, col, val))) {
        set_err("AMG recompute: %s", h->host.error.c_str());
        return LINA_GPU_ESETUP;
    }
    // the reference keeps the setup's signs and does not flip the new matrix
    if (h->host_only) return 0;
    if (!h->has_signs && !h->rmaps.empty()) {
        const int rc = refresh_values(h);
        if (rc != 1) return rc;  // done (0) or failed; 1: a pattern changed, rebuild
    }
    h->drop_graph();
    for (void* p : h->allocations) cudaFree(p);
    h->allocations.clear();
    h->dev_bytes = 0;
    // every pointer into the freed allocations is rebuilt on demand: the update maps and the Krylov
    // direction history (upload_hierarchy below re-creates the levels and the Krylov vectors)
    h->upd_built = false;
    h->upd_posQ = nullptr;
    h->kph = h->kqh = nullptr;
    h->hist_m = 0;
    h->Aorig = DCsr();
    h->rmaps.clear();
    h->rstage = nullptr;
    h->rstage_n = 0;
    h->rerr = nullptr;
    h->keep_maps = !h->has_signs;
    int rc = upload_hierarchy(h);
    h->keep_maps = false;
    if (rc) return rc;
    if (h->has_signs) rc = h->upload_csr(h->Aorig, csr_from(n, rowptr, col, val));
    return rc;
}

namespace {

// CSR entry -> layout position for a matrix uploaded by upload_csr (same layout choice)
std::vector<int> layout_positions(const lina::Csr& c, const std::vector<std::vector<int>>* groups) {
    if (csrv_lanes_for(c) > 0) {
        std::vector<int> pos(c.nnz());
        for (long k = 0; k < c.nnz(); k++) pos[k] = (int)k;
        return pos;
    }
    return make_sell(c, c.ncols > 0 ? c.ncols : c.n, groups).pos;
}

int build_update_maps(lina_gpu_amg* h) {
    const int f = h->depth - 1;
    const lina::HostLevel& F = h->host.lv[f];
    const lina::Csr& A = F.A;
    int rc;
    std::vector<int> posA = layout_positions(A, nullptr);
    if ((rc = h->upload(&h->upd_posA, posA.data(), posA.size()))) return rc;
    if (h->lv[f].A.q_val) {
        QuadHost Q;
        if (!make_quads(A, A.ncols > 0 ? A.ncols : A.n, Q)) {
            set_err("quad layout positions of the finest matrix could not be rebuilt");
            return LINA_GPU_ESETUP;
        }
        if ((rc = h->upload(&h->upd_posQ, Q.pos.data(), Q.pos.size()))) return rc;
    }
    {
        std::vector<int> colour;
        const int nc = lina::greedy_colouring(A, colour);
        std::vector<std::vector<int>> groups(nc);
        for (int i = 0; i < A.n; i++) groups[colour[i]].push_back(i);
        std::vector<int> posC = layout_positions(A, &groups);
        if ((rc = h->upload(&h->upd_posAcol, posC.data(), posC.size()))) return rc;
    }
    std::vector<int> diagpos(A.n, -1);
    std::vector<unsigned char> iso(A.n, 0);
    for (int i = 0; i < A.n; i++) {
        const bool skip = !F.labels.empty() && F.labels[i] == lina::kUndecided;
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++)
            if (A.col[p] == i && !skip) diagpos[i] = p;
        iso[i] = (!F.labels.empty() && F.labels[i] == lina::kIsolated) ? 1 : 0;
    }
    if ((rc = h->upload(&h->upd_diagpos, diagpos.data(), diagpos.size()))) return rc;
    if ((rc = h->upload(&h->upd_isolated, iso.data(), iso.size()))) return rc;
    if ((rc = h->upload(&h->upd_ptr, A.ptr.data(), A.ptr.size()))) return rc;
    if ((rc = h->alloc(&h->upd_val, std::max<long>(A.nnz(), 1)))) return rc;
    CK(cudaStreamSynchronize(h->stream));  // the host vectors above go out of scope
    h->upd_nnz = A.nnz();
    h->upd_built = true;
    return 0;
}

}  // namespace

int lina_gpu_amg_update_values(lina_gpu_amg* h, const double* val, int flags) {
    if (!h || h->host_only || !val) {
        set_err("lina_gpu_amg_update_values: invalid argument");
        return LINA_GPU_EINVAL;
    }
    if (h->depth < 2 || h->has_signs) {
        set_err("lina_gpu_amg_update_values: %s; use lina_gpu_amg_recompute",
                h->depth < 2 ? "a one-level hierarchy factorises its only matrix"
                             : "rows of the setup matrix were sign-flipped");
        return LINA_GPU_EINVAL;
    }
    int rc;
    if (!h->upd_built && (rc = build_update_maps(h))) return rc;
    const int f = h->depth - 1;
    DLevel& L = h->lv[f];
    const double* v = val;
    if (!(flags & LINA_PCG_DEVICE_PTRS)) {
        CK(cudaMemcpyAsync(h->upd_val, val, h->upd_nnz * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        v = h->upd_val;
    }
    go(update_values_kernel, grid_for(h->upd_nnz, kThreads), h->stream, h->upd_nnz, v, (const int*)h->upd_posA,
       (const int*)h->upd_posAcol, L.A.v64, L.A.v32, L.Acol.v64, L.Acol.v32, (const int*)h->upd_posQ,
       reinterpret_cast<float*>(L.A.q_val));
    go(update_diag_kernel, grid_for(L.n, kThreads), h->stream, L.n, v, (const int*)h->upd_ptr,
       (const int*)h->upd_diagpos, (const unsigned char*)h->upd_isolated, L.dinv64, L.dinv32, h->isoinv);
    if ((rc = stage_refresh(h, L))) return rc;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int lina_gpu_amg_destroy(lina_gpu_amg* h) {
    delete h;
    return 0;
}

int lina_gpu_amg_set_smoother(lina_gpu_amg* h, int smoother, double omega, int precision) {
    if (!h || (smoother != LINA_SMOOTHER_JACOBI && smoother != LINA_SMOOTHER_MC_SOR) ||
        (precision != LINA_PREC_FP64 && precision != LINA_PREC_MIXED)) {
        set_err("lina_gpu_amg_set_smoother: invalid argument");
        return LINA_GPU_EINVAL;
    }
    const bool new_omega = omega != h->opt.omega;
    h->opt.smoother = smoother;
    h->opt.omega = omega;
    h->opt.precision = precision;
    h->drop_graph();
    if (new_omega && !h->host_only) {
        int rc;
        for (DLevel& L : h->lv)
            if ((rc = stage_refresh(h, L))) return rc;
        CK(cudaStreamSynchronize(h->stream));
    }
    return 0;
}

int lina_gpu_amg_set_fcg_history(lina_gpu_amg* h, int m) {
    if (!h || m < 0 || m > kFcgMax) {
        set_err("lina_gpu_amg_set_fcg_history: m must be 0..%d", kFcgMax);
        return LINA_GPU_EINVAL;
    }
    h->fcg_m = m;
    h->drop_graph();
    return 0;
}

int lina_gpu_vcycle(lina_gpu_amg* h, const double* r_dev, double* z_dev) {
    if (!h || h->host_only || !r_dev || !z_dev) {
        set_err("lina_gpu_vcycle: invalid argument");
        return LINA_GPU_EINVAL;
    }
    const int n = h->lv[h->depth - 1].n;
    h->precondition(r_dev, z_dev, false);
    if (h->opt.precision == LINA_PREC_MIXED)
        go(convert_kernel<float, double>, grid_for(n, kThreads), h->stream, n, h->kz32, z_dev);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int lina_gpu_amg_solve(lina_gpu_amg* h, const double* F, double* X, double eps, int max_iter, int flags,
                       int* iterations, double* rel_residual) {
    if (!h || h->host_only || !F || !X || max_iter < 0) {
        set_err("lina_gpu_amg_solve: invalid argument");
        return LINA_GPU_EINVAL;
    }
    const int n = h->lv[h->depth - 1].n;
    const bool dev = (flags & LINA_PCG_DEVICE_PTRS) != 0;
    cudaStream_t st = h->stream;
    const int gv = grid_for(n, kThreads), gr = grid_red(n);
    double *b = h->kb, *x = h->kx, *r = h->kr;
    CK(cudaMemcpyAsync(b, F, n * sizeof(double), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(x, X, n * sizeof(double), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    if (h->has_signs) go(mul_kernel, gv, st, n, b, (const double*)h->signs);
    if (h->depth > 1) go(fix_isolated_kernel, gv, st, n, (const double*)b, (const double*)h->isoinv, x);
    const DCsr& A = h->lv[h->depth - 1].A;
    auto residual = [&]() -> double {
        h->csr<double, M_RESID>(A, x, r, b);
        go(norm2_kernel<double>, gr, st, n, (const double*)r, h->partials, h->ticket, h->sc);
        if (read_scalars(h)) return -1.0;
        return std::sqrt(h->sc_host->norm2);
    };
    const double r0 = residual();
    if (r0 < 0) return LINA_GPU_ECUDA;
    double rr = r0;
    int it = 0;
    // one V-cycle with initial guess x equals x + V(0, b - A x) for the linear smoothers used here
    while (r0 != 0.0 && std::fabs(rr / r0) > eps && it < max_iter) {
        h->precondition(r, h->kz, false, false);
        if (h->opt.precision == LINA_PREC_MIXED)
            go(add_kernel<float>, gv, st, n, x, (const float*)h->kz32);
        else
            go(add_kernel<double>, gv, st, n, x, (const double*)h->kz);
        rr = residual();
        if (rr < 0) return LINA_GPU_ECUDA;
        it++;
        if (!std::isfinite(rr)) break;
    }
    CK(cudaMemcpyAsync(X, x, n * sizeof(double), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (iterations) *iterations = it;
    if (rel_residual) *rel_residual = (r0 != 0.0) ? rr / r0 : 0.0;
    return std::isfinite(rr) ? 0 : LINA_GPU_EBREAKDOWN;
}

int lina_gpu_amg_fmg(lina_gpu_amg* h, const double* F, double* X, int flags, double* rel_residual) {
    if (!h || h->host_only || !F || !X) {
        set_err("lina_gpu_amg_fmg: invalid argument");
        return LINA_GPU_EINVAL;
    }
    const int n = h->lv[h->depth - 1].n;
    const bool dev = (flags & LINA_PCG_DEVICE_PTRS) != 0;
    cudaStream_t st = h->stream;
    const int gv = grid_for(n, kThreads), gr = grid_red(n);
    double *b = h->kb, *x = h->kx, *r = h->kr;
    CK(cudaMemcpyAsync(b, F, n * sizeof(double), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(x, X, n * sizeof(double), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    if (h->has_signs) go(mul_kernel, gv, st, n, b, (const double*)h->signs);
    const DCsr& A = h->lv[h->depth - 1].A;
    auto residual = [&]() -> double {
        h->csr<double, M_RESID>(A, x, r, b);
        go(norm2_kernel<double>, gr, st, n, (const double*)r, h->partials, h->ticket, h->sc);
        if (read_scalars(h)) return -1.0;
        return std::sqrt(h->sc_host->norm2);
    };
    const double r0 = residual();
    if (r0 < 0) return LINA_GPU_ECUDA;
    if (h->opt.precision == LINA_PREC_MIXED)
        h->fmg<float>(b, x);
    else
        h->fmg<double>(b, x);
    const double r1 = residual();
    if (r1 < 0) return LINA_GPU_ECUDA;
    CK(cudaMemcpyAsync(X, x, n * sizeof(double), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (rel_residual) *rel_residual = (r0 != 0.0) ? r1 / r0 : 0.0;
    return std::isfinite(r1) ? 0 : LINA_GPU_EBREAKDOWN;
}

int lina_gpu_spmv(lina_gpu_amg* h, int level, const double* x_dev, double* y_dev) {
    if (!h || h->host_only || level < 0 || level >= h->depth || !x_dev || !y_dev) {
        set_err("lina_gpu_spmv: invalid argument");
        return LINA_GPU_EINVAL;
    }
    const DCsr& A = h->lv[level].A;
    h->csr<double, M_SPMV>(A, x_dev, y_dev);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int lina_gpu_pcg(lina_gpu_amg* h, const double* b_in, double* x_out, double tol, int max_iter, int stop_rule,
                 int flags, lina_gpu_solve_info* info) {
    if (!h || h->host_only || !b_in || !x_out || max_iter < 1 ||
        (stop_rule != LINA_STOP_REFERENCE && stop_rule != LINA_STOP_RELATIVE)) {
        set_err("lina_gpu_pcg: invalid argument");
        return LINA_GPU_EINVAL;
    }
    lina_gpu_solve_info local{};
    lina_gpu_solve_info* inf = info ? info : &local;
    memset(inf, 0, sizeof *inf);
    const int n = h->lv[h->depth - 1].n;
    const bool dev = (flags & LINA_PCG_DEVICE_PTRS) != 0;
    const bool mixed = (h->opt.precision == LINA_PREC_MIXED);
    const bool time_it = (flags & LINA_PCG_TIME_KERNELS) != 0;
    h->beta_mode = (flags & LINA_PCG_BETA_FLEXIBLE) ? 1 : (flags & LINA_PCG_BETA_STANDARD) ? 0 : -1;
    h->ev_used = 0;
    cudaStream_t st = h->stream;
    double *b = h->kb, *x = h->kx, *r = h->kr, *z = h->kz;
    // inputs
    if (dev)
        CK(cudaMemcpyAsync(b, b_in, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    else
        CK(cudaMemcpyAsync(b, b_in, n * sizeof(double), cudaMemcpyHostToDevice, st));
    if (flags & LINA_PCG_USE_X0) {
        CK(cudaMemcpyAsync(x, x_out, n * sizeof(double), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                           st));
    } else {
        CK(cudaMemsetAsync(x, 0, n * sizeof(double), st));
    }
    CK(cudaMemsetAsync(h->sc, 0, sizeof(KScalars), st));
    const int gv = grid_for(n, kThreads);
    const int gr = grid_red(n);
    // ||b||
    go(norm2_kernel<double>, gr, st, n, b, h->partials, h->ticket, h->sc);
    if (read_scalars(h)) return LINA_GPU_ECUDA;
    double bnorm = std::sqrt(h->sc_host->norm2);
    double hscale = 1.0;
    if (flags & LINA_PCG_NORMALIZE) {
        hscale = (bnorm == 0.0) ? 1.0 : bnorm;
        double inv = 1.0 / hscale;
        CK(cudaMemcpyAsync(h->hscal, &inv, sizeof(double), cudaMemcpyHostToDevice, st));
        go(scale_kernel, gv, st, n, b, h->hscal, 0);
        go(scale_kernel, gv, st, n, x, h->hscal, 0);
        bnorm *= inv;
    }
    // r = b - A x
    const DCsr& A = h->krylov_matrix();
    h->csr<double, M_RESID>(A, x, r, b);
    // w = M^-1 r (kept as the first z)
    auto zptr_norm = [&]() {
        if (mixed)
            go(norm2_kernel<float>, gr, st, n, h->kz32, h->partials, h->ticket, h->sc);
        else
            go(norm2_kernel<double>, gr, st, n, z, h->partials, h->ticket, h->sc);
    };
    double r0 = 0.0;
    bool have_z = false;
    if (stop_rule == LINA_STOP_REFERENCE) {
        h->precondition(r, z, time_it);
        zptr_norm();
        CK(cudaGetLastError());
        if (read_scalars(h)) return LINA_GPU_ECUDA;
        r0 = std::sqrt(h->sc_host->norm2);
        have_z = true;
        if (r0 == 0.0) {
            inf->iterations = 0;
            goto finish;
        }
    } else {
        r0 = bnorm;
        if (r0 == 0.0) {
            CK(cudaMemsetAsync(x, 0, n * sizeof(double), st));
            inf->iterations = 0;
            goto finish;
        }
    }
    {
        // Iterations run either one by one from the host (kernel timing requested)
        // or as a captured CUDA graph whose while-loop node repeats the iteration
        // on the device until the residual test passes.
        const bool use_graph = !time_it && !(flags & LINA_PCG_HOST_LOOP);
        if (int rc = h->ensure_history()) return rc;
        int it = 0;
        int restarts = 0;
        int dev_iter = 0;  // the device's iteration counter (reset on restart)
        double rel = 0.0;
        for (;;) {
            if (use_graph && !have_z) {
                int rc = h->ensure_graph(n);
                if (rc) return rc;
                KScalars lim;
                lim.r0 = r0;
                lim.tol = tol;
                CK(cudaMemcpyAsync(&h->sc->r0, &lim.r0, sizeof(double), cudaMemcpyHostToDevice, st));
                CK(cudaMemcpyAsync(&h->sc->tol, &lim.tol, sizeof(double), cudaMemcpyHostToDevice, st));
                int maxit = dev_iter + (max_iter - it);
                CK(cudaMemcpyAsync(&h->sc->maxit, &maxit, sizeof(int), cudaMemcpyHostToDevice, st));
                CK(cudaGraphLaunch(h->gexec, st));
                if (read_scalars(h)) return LINA_GPU_ECUDA;
                int done = h->sc_host->iter - dev_iter;
                g_launches += (unsigned long long)done * (unsigned long long)h->g_kernels;
                it += done;
                dev_iter = h->sc_host->iter;
            } else {
                h->issue_iteration(n, !have_z, time_it);
                have_z = false;
                CK(cudaGetLastError());
                if (read_scalars(h)) return LINA_GPU_ECUDA;
                it++;
                dev_iter = h->sc_host->iter;
            }
            rel = std::sqrt(h->sc_host->rr) / r0;
            if (!std::isfinite(rel)) {
                inf->status = LINA_GPU_EBREAKDOWN;
                break;
            }
            bool converged = rel <= tol;
            if (converged && stop_rule == LINA_STOP_RELATIVE && restarts < 8) {
                // confirm on the true residual; restart the recurrence from it if needed
                true_residual(h, b, x);
                if (read_scalars(h)) return LINA_GPU_ECUDA;
                double trel = std::sqrt(h->sc_host->norm2) / r0;
                if (trel > tol) {
                    CK(cudaMemcpyAsync(r, h->kt, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
                    int zero = 0;
                    CK(cudaMemcpyAsync(&h->sc->iter, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
                    dev_iter = 0;
                    restarts++;
                    converged = false;
                }
            }
            if (converged || it >= max_iter) break;
        }
        inf->iterations = it;
        inf->restarts = restarts;
        inf->rel_residual = rel;
        if (inf->status == 0 && rel > tol) inf->status = LINA_GPU_ENOCONV;
    }
finish:
    if ((flags & LINA_PCG_FINAL_PRECON) && r0 != 0.0 && stop_rule == LINA_STOP_REFERENCE) {
        h->precondition(r, z, false);
        zptr_norm();
        if (read_scalars(h)) return LINA_GPU_ECUDA;
        inf->pcg_residuum = std::sqrt(h->sc_host->norm2) / r0;
    }
    true_residual(h, b, x);
    if (read_scalars(h)) return LINA_GPU_ECUDA;
    inf->true_rel_residual = (bnorm > 0) ? std::sqrt(h->sc_host->norm2) / bnorm : 0.0;
    // the relative rule is met only when the true residual meets it (after the restarts are used up
    // the recurrence may claim more than the arithmetic can deliver)
    if (stop_rule == LINA_STOP_RELATIVE && inf->status == 0 && r0 > 0.0 && std::sqrt(h->sc_host->norm2) / r0 > tol)
        inf->status = LINA_GPU_ENOCONV;
    if (flags & LINA_PCG_NORMALIZE) {
        CK(cudaMemcpyAsync(h->hscal, &hscale, sizeof(double), cudaMemcpyHostToDevice, st));
        go(scale_kernel, gv, st, n, x, h->hscal, 0);
    }
    if (dev)
        CK(cudaMemcpyAsync(x_out, x, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    else
        CK(cudaMemcpyAsync(x_out, x, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (time_it && h->ev_used >= 2) {
        double tot = 0.0;
        for (int k = 0; k + 1 < h->ev_used; k += 2) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, h->ev_pool[k], h->ev_pool[k + 1]);
            tot += ms;
        }
        inf->smoother_ms = tot;
        inf->smoother_launches = h->ev_used / 2;
        const DLevel& L = h->lv[h->timed_level];
        double nnz = (double)L.A.nnz, nn = (double)L.n;
        inf->timed_level = h->timed_level;
        inf->timed_rows = L.n;
        inf->timed_entries = L.A.nnz;
        // a stored entry: its value and its column index (2 bytes in the 16-bit SELL layout); the
        // row structure as a CSR row pointer; x, b, 1/a_ii read and y written once
        const DCsr& sm = h->opt.smoother == LINA_SMOOTHER_JACOBI ? L.A : L.Acol;
        const double ib = (mixed && sm.col16) ? 2.0 : 4.0;
        const double sweep = mixed ? ((4 + ib) * nnz + 4 * (nn + 1) + 16 * nn) : ((8 + ib) * nnz + 4 * (nn + 1) + 32 * nn);
        if (h->opt.smoother == LINA_SMOOTHER_JACOBI)
            inf->smoother_bytes = sweep;
        else  // one colour launch: average share of the sweep
            inf->smoother_bytes = sweep / L.ncolours;
    }
    return inf->status;
}

int lina_gpu_timer_begin(lina_gpu_amg* h) {
    if (!h || h->host_only) return LINA_GPU_EINVAL;
    if (!h->tm0) {
        CK(cudaEventCreate(&h->tm0));
        CK(cudaEventCreate(&h->tm1));
    }
    CK(cudaEventRecord(h->tm0, h->stream));
    return 0;
}

int lina_gpu_timer_end(lina_gpu_amg* h, double* ms) {
    if (!h || h->host_only || !h->tm0 || !ms) return LINA_GPU_EINVAL;
    CK(cudaEventRecord(h->tm1, h->stream));
    CK(cudaEventSynchronize(h->tm1));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, h->tm0, h->tm1));
    *ms = f;
    return 0;
}

unsigned long long lina_gpu_launches(void) { return g_launches; }

void* lina_gpu_malloc_host(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) {
        set_err("cudaMallocHost(%zu) failed", bytes);
        return nullptr;
    }
    return p;
}

int lina_gpu_free_host(void* p) {
    CK(cudaFreeHost(p));
    return 0;
}

// ------------------------------------------------------------ single matrices
// A standalone matrix on the device (SELL-32, FP64 and FP32 values) with the
// same kernels as the hierarchy levels; it reuses the hierarchy machinery with
// a one-level, setup-free handle.
struct lina_gpu_matrix {
    lina_gpu_amg* h = nullptr;
    DCsr A;
    double* dinv64 = nullptr;
    float* dinv32 = nullptr;
    // for lina_gpu_matrix_update_values: stored position of each CSR entry (host until first use),
    // the last diagonal entry of each row, staging for new values
    long nnz = 0;
    std::vector<int> pos_host, diag_host, qpos_host;
    int *pos = nullptr, *diagpos = nullptr, *qpos = nullptr;
    double* stage = nullptr;
};

namespace {

// new values on the stored pattern: SELL (or CSR) values in both precisions and the inverse diagonal
// (the last diagonal entry of a row, 0 where it is absent or zero, as at creation)
__global__ void matrix_values_kernel(long nnz, const double* __restrict__ val, const int* __restrict__ pos,
                                     double* __restrict__ v64, float* __restrict__ v32, const int* __restrict__ qpos,
                                     float* __restrict__ q32) {
    pdl_wait();
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x) {
        const int p = pos ? pos[k] : (int)k;
        if (p >= 0) {
            v64[p] = val[k];
            v32[p] = float(val[k]);
        }
        if (qpos) {
            const int q = qpos[k];
            if (q >= 0) q32[q] = float(val[k]);
        }
    }
}

__global__ void matrix_dinv_kernel(int n, const double* __restrict__ val, const int* __restrict__ diagpos,
                                   double* __restrict__ d64, float* __restrict__ d32) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = diagpos[i];
        const double d = (p >= 0 && val[p] != 0.0) ? 1.0 / val[p] : 0.0;
        d64[i] = d;
        d32[i] = float(d);
    }
}

}  // namespace

int lina_gpu_matrix_create(int n, int ncols, const int* rowptr, const int* col, const double* val,
                           lina_gpu_matrix** out) {
    if (!out || n <= 0 || ncols <= 0 || !rowptr || !col || !val || rowptr[0] != 0) {
        set_err("lina_gpu_matrix_create: invalid argument");
        return LINA_GPU_EINVAL;
    }
    for (int i = 0; i < n; i++)
        if (rowptr[i + 1] < rowptr[i]) {
            set_err("lina_gpu_matrix_create: row pointers decrease at row %d", i);
            return LINA_GPU_EINVAL;
        }
    *out = nullptr;
    lina_gpu_matrix* m = new lina_gpu_matrix();
    m->h = new lina_gpu_amg();
    lina_gpu_amg* h = m->h;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_err("cudaStreamCreate failed");
        delete h;
        delete m;
        return LINA_GPU_ECUDA;
    }
    lina::Csr c;
    c.n = n;
    c.ncols = ncols;
    c.ptr.assign(rowptr, rowptr + n + 1);
    c.col.resize(rowptr[n]);
    c.val.resize(rowptr[n]);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        std::copy(col + rowptr[i], col + rowptr[i + 1], c.col.begin() + rowptr[i]);
        std::copy(val + rowptr[i], val + rowptr[i + 1], c.val.begin() + rowptr[i]);
    }
    std::vector<double> dinv(n, 0.0);
    std::vector<float> dinv32(n);
    m->nnz = rowptr[n];
    m->diag_host.assign(n, -1);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        for (int p = c.ptr[i]; p < c.ptr[i + 1]; p++)
            if (c.col[p] == i) {
                m->diag_host[i] = p;
                if (c.val[p] != 0.0) dinv[i] = 1.0 / c.val[p];
            }
        dinv32[i] = (float)dinv[i];
    }
    int rc = h->upload_csr(m->A, c, nullptr, &m->pos_host, &m->qpos_host);
    if (!rc) rc = h->upload(&m->dinv64, dinv.data(), dinv.size());
    if (!rc) rc = h->upload(&m->dinv32, dinv32.data(), dinv32.size());
    if (!rc) rc = h->alloc(&h->partials, 2 * kMaxBlocks);
    if (!rc) rc = h->alloc(&h->ticket, 4);
    if (!rc) rc = h->alloc(&h->sc, 1);
    if (!rc && cudaMemsetAsync(h->ticket, 0, 4 * sizeof(unsigned), h->stream) != cudaSuccess) rc = LINA_GPU_ECUDA;
    if (!rc && cudaMemsetAsync(h->sc, 0, sizeof(KScalars), h->stream) != cudaSuccess) rc = LINA_GPU_ECUDA;
    if (!rc && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = LINA_GPU_ECUDA;
    if (rc) {
        delete h;
        delete m;
        return rc;
    }
    *out = m;
    return 0;
}

int lina_gpu_matrix_update_values(lina_gpu_matrix* m, const double* val, int flags) {
    if (!m || !val) {
        set_err("lina_gpu_matrix_update_values: invalid argument");
        return LINA_GPU_EINVAL;
    }
    lina_gpu_amg* h = m->h;
    int rc = 0;
    if (!m->diagpos) {
        if (!m->pos_host.empty()) rc = h->upload(&m->pos, m->pos_host.data(), m->pos_host.size());
        if (!rc && !m->qpos_host.empty()) rc = h->upload(&m->qpos, m->qpos_host.data(), m->qpos_host.size());
        if (!rc) rc = h->upload(&m->diagpos, m->diag_host.data(), m->diag_host.size());
        if (!rc && !(flags & LINA_PCG_DEVICE_PTRS)) rc = h->alloc(&m->stage, (size_t)m->nnz);
        if (!rc && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = LINA_GPU_ECUDA;
        if (rc) return rc;
        m->pos_host = std::vector<int>();
        m->qpos_host = std::vector<int>();
    }
    const double* v = val;
    if (!(flags & LINA_PCG_DEVICE_PTRS)) {
        if (!m->stage && (rc = h->alloc(&m->stage, (size_t)m->nnz))) return rc;
        CK(cudaMemcpyAsync(m->stage, val, (size_t)m->nnz * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        v = m->stage;
    }
    go(matrix_values_kernel, grid_for(m->nnz, kThreads), h->stream, m->nnz, v, (const int*)m->pos, m->A.v64,
       m->A.v32, (const int*)m->qpos, reinterpret_cast<float*>(m->A.q_val));
    go(matrix_dinv_kernel, grid_for(m->A.n, kThreads), h->stream, m->A.n, v, (const int*)m->diagpos, m->dinv64,
       m->dinv32);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int lina_gpu_matrix_destroy(lina_gpu_matrix* m) {
    if (m) {
        delete m->h;
        delete m;
    }
    return 0;
}

int lina_gpu_matrix_spmv(lina_gpu_matrix* m, int precision, const void* x_dev, void* y_dev) {
    if (!m || !x_dev || !y_dev) {
        set_err("lina_gpu_matrix_spmv: invalid argument");
        return LINA_GPU_EINVAL;
    }
    if (precision == LINA_PREC_MIXED)
        m->h->csr<float, M_SPMV>(m->A, (const float*)x_dev, (float*)y_dev);
    else
        m->h->csr<double, M_SPMV>(m->A, (const double*)x_dev, (double*)y_dev);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(m->h->stream));
    return 0;
}

int lina_gpu_matrix_jacobi(lina_gpu_matrix* m, int precision, double omega, int sweeps, const void* b_dev,
                           void* x_dev, void* tmp_dev) {
    if (!m || !b_dev || !x_dev || !tmp_dev || sweeps < 0) {
        set_err("lina_gpu_matrix_jacobi: invalid argument");
        return LINA_GPU_EINVAL;
    }
    for (int k = 0; k < sweeps; k++) {
        const bool even = (k % 2 == 0);
        if (precision == LINA_PREC_MIXED) {
            const float* xi = (const float*)(even ? x_dev : tmp_dev);
            float* xo = (float*)(even ? tmp_dev : x_dev);
            m->h->csr<float, M_JACOBI>(m->A, xi, xo, (const float*)b_dev, m->dinv32, (float)omega);
        } else {
            const double* xi = (const double*)(even ? x_dev : tmp_dev);
            double* xo = (double*)(even ? tmp_dev : x_dev);
            m->h->csr<double, M_JACOBI>(m->A, xi, xo, (const double*)b_dev, m->dinv64, omega);
        }
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(m->h->stream));
    return 0;
}

long lina_gpu_matrix_padded_entries(const lina_gpu_matrix* m) { return m ? m->A.padded : 0; }

int lina_gpu_matrix_rows(const lina_gpu_matrix* m) { return m ? m->A.n : 0; }

int lina_gpu_matrix_index_bits(const lina_gpu_matrix* m) {
    if (!m || m->A.lanes > 0) return 0;
    return (m->A.col16 || m->A.q_val) ? 16 : 32;
}

int lina_gpu_amg_depth(const lina_gpu_amg* h) { return h ? h->depth : 0; }

int lina_gpu_level_index_bits(const lina_gpu_amg* h, int level, int* A_bits, int* P_bits, int* R_bits) {
    if (!h || h->host_only || level < 0 || level >= (int)h->lv.size()) return LINA_GPU_EINVAL;
    auto bits = [](const DCsr& d) { return d.lanes > 0 || !d.col ? 0 : ((d.col16 || d.q_val) ? 16 : 32); };
    const DLevel& L = h->lv[level];
    if (A_bits) *A_bits = bits(L.A);
    if (P_bits) *P_bits = level > 0 ? bits(L.P) : 0;
    if (R_bits) *R_bits = level > 0 ? bits(L.R) : 0;
    return 0;
}

int lina_gpu_level_sizes(const lina_gpu_amg* h, int level, int* n, long* nnz_A, long* nnz_P, long* nnz_R,
                         int* n_colours) {
    if (!h || level < 0 || level >= h->depth) return LINA_GPU_EINVAL;
    const lina::HostLevel& L = h->host.lv[level];
    if (n) *n = L.A.n;
    if (nnz_A) *nnz_A = (long)L.A.nnz();
    if (nnz_P) *nnz_P = (long)L.P.nnz();
    if (nnz_R) *nnz_R = (long)L.R.nnz();
    if (n_colours) *n_colours = (level < (int)h->lv.size()) ? h->lv[level].ncolours : 0;
    return 0;
}

int lina_gpu_level_export(const lina_gpu_amg* h, int level, int* labels, int* A_ptr, int* A_col, double* A_val,
                          int* P_ptr, int* P_col, double* P_val, int* R_ptr, int* R_col, double* R_val) {
    if (!h || level < 0 || level >= h->depth) return LINA_GPU_EINVAL;
    const lina::HostLevel& L = h->host.lv[level];
    auto cp = [](const lina::Csr& c, int* pp, int* cc, double* vv) {
        if (pp) std::copy(c.ptr.begin(), c.ptr.end(), pp);
        if (cc) std::copy(c.col.begin(), c.col.end(), cc);
        if (vv) std::copy(c.val.begin(), c.val.end(), vv);
    };
    if (labels && !L.labels.empty()) std::copy(L.labels.begin(), L.labels.end(), labels);
    cp(L.A, A_ptr, A_col, A_val);
    if (level > 0) {
        cp(L.P, P_ptr, P_col, P_val);
        cp(L.R, R_ptr, R_col, R_val);
    }
    return 0;
}

int lina_gpu_level_colours(const lina_gpu_amg* h, int level, int* colour) {
    if (!h || level < 0 || level >= h->depth || !colour) return LINA_GPU_EINVAL;
    std::vector<int> c;
    lina::greedy_colouring(h->host.lv[level].A, c);
    std::copy(c.begin(), c.end(), colour);
    return 0;
}

int lina_gpu_coarse_block_size(const lina_gpu_amg* h) { return h ? (int)h->host.coarse.block_rows.size() : 0; }

long lina_gpu_amg_device_bytes(const lina_gpu_amg* h) { return h ? h->dev_bytes : 0; }

void* lina_gpu_malloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
        set_err("cudaMalloc(%zu) failed", bytes);
        return nullptr;
    }
    return p;
}

int lina_gpu_free(void* p) {
    CK(cudaFree(p));
    return 0;
}

int lina_gpu_memcpy_h2d(void* dst, const void* src, size_t bytes) {
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return 0;
}

int lina_gpu_memcpy_d2h(void* dst, const void* src, size_t bytes) {
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return 0;
}

int lina_gpu_synchronize(void) {
    CK(cudaDeviceSynchronize());
    return 0;
}

}  // extern "C"

// =================================================================== batched solves
// Many independent systems in one CUDA graph: for every system a branch of
//   start (x = 0, r = b, ||b||, and ||M^-1 b|| for the reference's rule)
//   -> a one-thread kernel that sets the loop's limits and whether it runs at all
//   -> a while-loop node whose body is the PCG iteration of lina_gpu_pcg
//   -> the true residual ||b - A x||.
// The branches share nothing (each system has its own vectors, reductions and scalars), so one
// launch runs them all concurrently: the small systems, which are bound by launch and memory
// latency, overlap one another and the large ones.
namespace {

struct BatchLimits {
    double tol;
    int maxit;
    int pad;
};

__global__ void save_norm_kernel(KScalars* sc) {
    pdl_wait();
    sc->aux = sc->norm2;
}

// sc->norm2 holds r0^2 (||b||^2 or ||M^-1 b||^2); the loop runs when r0 is a positive number
__global__ void batch_start_kernel(cudaGraphConditionalHandle hd, KScalars* sc, const BatchLimits* lim) {
    pdl_wait();
    const double r0 = sqrt(sc->norm2);
    sc->r0 = r0;
    sc->tol = lim->tol;
    sc->maxit = lim->maxit;
    sc->iter = 0;
    cudaGraphSetConditional(hd, (r0 > 0.0 && isfinite(r0) && lim->maxit > 0) ? 1u : 0u);
}

}  // namespace

struct lina_gpu_batch {
    std::vector<lina_gpu_amg*> sys;
    int stop_rule = LINA_STOP_RELATIVE;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    BatchLimits* lim = nullptr;       // device
    BatchLimits* lim_host = nullptr;  // pinned
    KScalars* sc_host = nullptr;      // pinned, one per system
    std::vector<long> k_start, k_iter, k_finish;  // kernels per branch part
    ~lina_gpu_batch() {
        if (stream) cudaStreamSynchronize(stream);
        if (exec) cudaGraphExecDestroy(exec);
        if (lim) cudaFree(lim);
        if (lim_host) cudaFreeHost(lim_host);
        if (sc_host) cudaFreeHost(sc_host);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// capture the work `f` issues on h's stream as a graph (counting its kernels)
template <typename F>
int capture_on(lina_gpu_amg* h, cudaGraph_t* g, long* kernels, F f) {
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed));
    const unsigned long long before = g_launches;
    f();
    *kernels = (long)(g_launches - before);
    g_launches = before;
    cudaError_t e = cudaStreamEndCapture(h->stream, g);
    if (e != cudaSuccess) {
        set_err("batch capture failed: %s", cudaGetErrorString(e));
        return LINA_GPU_ECUDA;
    }
    return 0;
}

int build_batch_graph(lina_gpu_batch* B) {
    cudaGraph_t G = nullptr;
    CK(cudaGraphCreate(&G, 0));
    int rc = 0;
    for (size_t s = 0; s < B->sys.size() && !rc; s++) {
        lina_gpu_amg* h = B->sys[s];
        const int n = h->lv[h->depth - 1].n;
        const bool mixed = (h->opt.precision == LINA_PREC_MIXED);
        const int gr = grid_red(n);
        h->beta_mode = -1;
        if ((rc = h->ensure_history())) break;
        cudaGraph_t gstart = nullptr, gfin = nullptr;
        rc = capture_on(h, &gstart, &B->k_start[s], [&] {
            cudaMemsetAsync(h->kx, 0, (size_t)n * sizeof(double), h->stream);
            cudaMemsetAsync(h->sc, 0, sizeof(KScalars), h->stream);
            cudaMemcpyAsync(h->kr, h->kb, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream);
            go(norm2_kernel<double>, gr, h->stream, n, (const double*)h->kb, h->partials, h->ticket, h->sc);
            g_launches++;
            save_norm_kernel<<<1, 1, 0, h->stream>>>(h->sc);
            if (B->stop_rule == LINA_STOP_REFERENCE) {
                h->precondition(h->kr, h->kz, false);
                if (mixed)
                    go(norm2_kernel<float>, gr, h->stream, n, (const float*)h->kz32, h->partials, h->ticket, h->sc);
                else
                    go(norm2_kernel<double>, gr, h->stream, n, (const double*)h->kz, h->partials, h->ticket, h->sc);
            }
        });
        if (!rc)
            rc = capture_on(h, &gfin, &B->k_finish[s], [&] { true_residual(h, h->kb, h->kx); });
        cudaGraphNode_t n_start = nullptr, n_cond = nullptr, n_loop = nullptr, n_fin = nullptr;
        cudaGraphConditionalHandle hd = 0;
        cudaError_t e = rc ? cudaErrorUnknown : cudaGraphAddChildGraphNode(&n_start, G, nullptr, 0, gstart);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hd, G, 0, cudaGraphCondAssignDefault);
        if (e == cudaSuccess) {
            void* args[] = {(void*)&hd, (void*)&h->sc, (void*)&B->lim};
            cudaKernelNodeParams kp = {};
            kp.func = (void*)batch_start_kernel;
            kp.gridDim = dim3(1);
            kp.blockDim = dim3(1);
            kp.kernelParams = args;
            e = cudaGraphAddKernelNode(&n_cond, G, &n_start, 1, &kp);
        }
        cudaGraphNodeParams cp = {};
        if (e == cudaSuccess) {
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = hd;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            e = cudaGraphAddNode(&n_loop, G, &n_cond, nullptr, 1, &cp);
        }
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(h->stream, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            const unsigned long long before = g_launches;
            h->beta_mode = -1;  // the precision's default recurrence
            h->issue_iteration(n, true, false);
            loop_cond_kernel<<<1, 1, 0, h->stream>>>(hd, h->sc);
            B->k_iter[s] = (long)(g_launches - before) + 1;
            g_launches = before;
            cudaGraph_t body = nullptr;
            e = cudaStreamEndCapture(h->stream, &body);
        }
        if (e == cudaSuccess) e = cudaGraphAddChildGraphNode(&n_fin, G, &n_loop, 1, gfin);
        if (gstart) cudaGraphDestroy(gstart);
        if (gfin) cudaGraphDestroy(gfin);
        if (!rc && e != cudaSuccess) {
            set_err("batch graph construction failed: %s", cudaGetErrorString(e));
            rc = LINA_GPU_ECUDA;
        }
    }
    if (!rc) {
        cudaError_t e = cudaGraphInstantiate(&B->exec, G, 0);
        if (e != cudaSuccess) {
            B->exec = nullptr;
            set_err("batch graph instantiation failed: %s", cudaGetErrorString(e));
            rc = LINA_GPU_ECUDA;
        }
    }
    cudaGraphDestroy(G);
    return rc;
}

}  // namespace

extern "C" {

int lina_gpu_batch_create(int count, lina_gpu_amg* const* systems, int stop_rule, lina_gpu_batch** out) {
    if (!out || count < 1 || !systems || (stop_rule != LINA_STOP_REFERENCE && stop_rule != LINA_STOP_RELATIVE)) {
        set_err("lina_gpu_batch_create: invalid argument");
        return LINA_GPU_EINVAL;
    }
    *out = nullptr;
    for (int i = 0; i < count; i++) {
        if (!systems[i] || systems[i]->host_only) {
            set_err("lina_gpu_batch_create: system %d is not a device hierarchy", i);
            return LINA_GPU_EINVAL;
        }
        for (int j = 0; j < i; j++)
            if (systems[j] == systems[i]) {
                set_err("lina_gpu_batch_create: system %d appears twice", i);
                return LINA_GPU_EINVAL;
            }
    }
    lina_gpu_batch* B = new lina_gpu_batch();
    B->sys.assign(systems, systems + count);
    B->stop_rule = stop_rule;
    B->k_start.assign(count, 0);
    B->k_iter.assign(count, 0);
    B->k_finish.assign(count, 0);
    if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&B->lim, sizeof(BatchLimits)) != cudaSuccess ||
        cudaMallocHost(&B->lim_host, sizeof(BatchLimits)) != cudaSuccess ||
        cudaMallocHost(&B->sc_host, (size_t)count * sizeof(KScalars)) != cudaSuccess) {
        set_err("lina_gpu_batch_create: allocation failed");
        delete B;
        return LINA_GPU_ECUDA;
    }
    // every system's hierarchy and vectors are ready before the capture
    for (lina_gpu_amg* h : B->sys)
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
            set_err("lina_gpu_batch_create: a system's stream failed");
            delete B;
            return LINA_GPU_ECUDA;
        }
    int rc = build_batch_graph(B);
    if (rc) {
        delete B;
        return rc;
    }
    *out = B;
    return 0;
}

int lina_gpu_batch_solve(lina_gpu_batch* B, const double* const* b, double* const* x, double tol, int max_iter,
                         int flags, lina_gpu_solve_info* infos) {
    if (!B || !b || !x || max_iter < 1) {
        set_err("lina_gpu_batch_solve: invalid argument");
        return LINA_GPU_EINVAL;
    }
    const int count = (int)B->sys.size();
    for (int i = 0; i < count; i++)
        if (!b[i] || !x[i]) {
            set_err("lina_gpu_batch_solve: missing vector of system %d", i);
            return LINA_GPU_EINVAL;
        }
    const bool dev = (flags & LINA_PCG_DEVICE_PTRS) != 0;
    cudaStream_t st = B->stream;
    B->lim_host->tol = tol;
    B->lim_host->maxit = max_iter;
    CK(cudaMemcpyAsync(B->lim, B->lim_host, sizeof(BatchLimits), cudaMemcpyHostToDevice, st));
    for (int i = 0; i < count; i++) {
        lina_gpu_amg* h = B->sys[i];
        const int n = h->lv[h->depth - 1].n;
        CK(cudaMemcpyAsync(h->kb, b[i], (size_t)n * sizeof(double),
                           dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    }
    CK(cudaGraphLaunch(B->exec, st));
    for (int i = 0; i < count; i++) {
        lina_gpu_amg* h = B->sys[i];
        const int n = h->lv[h->depth - 1].n;
        CK(cudaMemcpyAsync(B->sc_host + i, h->sc, sizeof(KScalars), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(x[i], h->kx, (size_t)n * sizeof(double),
                           dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    int rc = 0;
    for (int i = 0; i < count; i++) {
        const KScalars& k = B->sc_host[i];
        g_launches += (unsigned long long)(B->k_start[i] + 1 + B->k_finish[i] + (long)k.iter * B->k_iter[i]);
        lina_gpu_solve_info inf{};
        const double bnorm = std::sqrt(k.aux);
        inf.iterations = k.iter;
        inf.rel_residual = k.r0 > 0.0 ? std::sqrt(k.rr) / k.r0 : 0.0;
        inf.true_rel_residual = bnorm > 0.0 ? std::sqrt(k.norm2) / bnorm : 0.0;
        if (k.r0 > 0.0 && !std::isfinite(inf.rel_residual))
            inf.status = LINA_GPU_EBREAKDOWN;
        else if (inf.rel_residual > tol)
            inf.status = LINA_GPU_ENOCONV;
        // the relative rule is met only when the true residual meets it: otherwise the solve goes on
        // from the batch's x with the single-system path (which restarts on the true residual)
        if (B->stop_rule == LINA_STOP_RELATIVE && inf.status == 0 && inf.true_rel_residual > tol &&
            inf.iterations < max_iter) {
            lina_gpu_solve_info more{};
            int r = lina_gpu_pcg(B->sys[i], b[i], x[i], tol, max_iter - inf.iterations, LINA_STOP_RELATIVE,
                                 (flags & LINA_PCG_DEVICE_PTRS) | LINA_PCG_USE_X0, &more);
            if (r && r != LINA_GPU_ENOCONV) return r;
            inf.iterations += more.iterations;
            inf.rel_residual = more.true_rel_residual;
            inf.true_rel_residual = more.true_rel_residual;
            inf.status = more.status;
        } else if (B->stop_rule == LINA_STOP_RELATIVE && inf.status == 0 && inf.true_rel_residual > tol) {
            inf.status = LINA_GPU_ENOCONV;
        }
        if (infos) infos[i] = inf;
        if (inf.status && !rc) rc = inf.status == LINA_GPU_ENOCONV ? LINA_GPU_ENOCONV : inf.status;
    }
    return rc;
}

int lina_gpu_batch_size(const lina_gpu_batch* B) { return B ? (int)B->sys.size() : 0; }

int lina_gpu_batch_destroy(lina_gpu_batch* B) {
    delete B;
    return 0;
}

}  // extern "C"

// =================================================================== segmented batched solves
// Many independent systems solved as one: every level of one hierarchy is the block-diagonal
// concatenation of the systems' levels (a segmented CSR: system i's rows, and its columns, follow the
// rows of systems 0..i-1), so each kernel of the V-cycle streams all systems' rows in one launch.  A
// system whose hierarchy is shallower than the deepest one is padded below its coarsest level with
// copies of that level (P = R = I); a V-cycle returns there the exact coarse solution, as the system's
// own V-cycle does, and the padded levels cost a few sweeps of its small coarsest matrix.  The coarsest
// level is solved block by block with each system's own dense inverse.  The Krylov loop is FCG(m) per
// system: its reductions are segmented (fixed chunks of rows that never straddle two systems, summed
// per system in chunk order), each system has its own scalars, stops at its own tolerance and then
// keeps x and r while the others continue; one CUDA graph with a device-side while loop runs until
// every system has stopped.
namespace {

constexpr int kSegChunk = 4096;  // rows per task of the segmented kernels

struct SegScalars {
    double s, s_old, pq, alpha, rr, r0, tol, tnorm2;
    double tj[kFcgMax], pqh[kFcgMax], cj[kFcgMax];
    int iter, base, active, maxit, status, pad;
};

enum { SEG_DOT = 0, SEG_PQ = 1, SEG_RR = 2, SEG_NORM_B = 3, SEG_NORM_T = 4 };

// the block's sums of v[0..NV) into out[0..NV)
template <int NV>
__device__ void seg_block_sums(const double (&v)[NV], double* out) {
    __shared__ double sm[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        const double x = warp_sum(v[k]);
        if (lane == 0) sm[k][wid] = x;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double x = (lane < nw) ? sm[k][lane] : 0.0;
            x = warp_sum(x);
            if (lane == 0) out[k] = x;
        }
    }
    __syncthreads();  // sm is reused by the block's next task
}

// s = r.z and t_j = z.q_{k-j} (j = 1..min(k - base, M)) per task of an active system
template <typename TZ, int M>
__global__ void __launch_bounds__(kThreads) seg_fcg_dot_kernel(int ntask, const int4* __restrict__ task, long n,
                                                               const double* __restrict__ r,
                                                               const TZ* __restrict__ z, const double* __restrict__ qh,
                                                               const SegScalars* __restrict__ sc,
                                                               double* __restrict__ part) {
    pdl_wait();
    for (int t = blockIdx.x; t < ntask; t += gridDim.x) {
        const int4 tk = task[t];
        double v[M + 1];
#pragma unroll
        for (int j = 0; j <= M; j++) v[j] = 0.0;
        if (sc[tk.x].active) {
            const int k = sc[tk.x].iter;
            const int nprev = min(k - sc[tk.x].base, M);
            const double* qs[M];
#pragma unroll
            for (int j = 1; j <= M; j++) qs[j - 1] = qh + (size_t)((k - j + M * kFcgMax) % M) * n;
            for (long i = tk.y + threadIdx.x; i < tk.z; i += blockDim.x) {
                const double zi = double(z[i]);
                v[0] += r[i] * zi;
#pragma unroll
                for (int j = 1; j <= M; j++)
                    if (j <= nprev) v[j] += zi * qs[j - 1][i];
            }
        }
        seg_block_sums<M + 1>(v, part + (size_t)t * (M + 1));
    }
}

// p = z - sum_j c_j p_{k-j} per task of an active system
template <typename TZ, int M>
__global__ void __launch_bounds__(kThreads) seg_fcg_update_p_kernel(int ntask, const int4* __restrict__ task, long n,
                                                                    const TZ* __restrict__ z,
                                                                    const double* __restrict__ ph,
                                                                    double* __restrict__ p,
                                                                    const SegScalars* __restrict__ sc) {
    pdl_wait();
    for (int t = blockIdx.x; t < ntask; t += gridDim.x) {
        const int4 tk = task[t];
        if (!sc[tk.x].active) continue;
        const int k = sc[tk.x].iter;
        const int nprev = min(k - sc[tk.x].base, M);
        double c[M];
        const double* ps[M];
#pragma unroll
        for (int j = 1; j <= M; j++) {
            c[j - 1] = sc[tk.x].cj[j - 1];
            ps[j - 1] = ph + (size_t)((k - j + M * kFcgMax) % M) * n;
        }
        for (long i = tk.y + threadIdx.x; i < tk.z; i += blockDim.x) {
            double pi = double(z[i]);
#pragma unroll
            for (int j = 1; j <= M; j++)
                if (j <= nprev) pi -= c[j - 1] * ps[j - 1][i];
            p[i] = pi;
        }
    }
}

// a.b per task
__global__ void __launch_bounds__(kThreads) seg_dot_kernel(int ntask, const int4* __restrict__ task,
                                                           const double* __restrict__ a, const double* __restrict__ b,
                                                           double* __restrict__ part) {
    pdl_wait();
    for (int t = blockIdx.x; t < ntask; t += gridDim.x) {
        const int4 tk = task[t];
        double v[1] = {0.0};
        for (long i = tk.y + threadIdx.x; i < tk.z; i += blockDim.x) v[0] += a[i] * b[i];
        seg_block_sums<1>(v, part + t);
    }
}

// x += alpha p, r -= alpha q, ring slot (iter mod M) <- p, q for active systems; r.r per task
template <int M>
__global__ void __launch_bounds__(kThreads) seg_update_xr_kernel(int ntask, const int4* __restrict__ task, long n,
                                                                 double* __restrict__ x, double* __restrict__ r,
                                                                 const double* __restrict__ p,
                                                                 const double* __restrict__ q, double* __restrict__ ph,
                                                                 double* __restrict__ qh,
                                                                 const SegScalars* __restrict__ sc,
                                                                 double* __restrict__ part) {
    pdl_wait();
    for (int t = blockIdx.x; t < ntask; t += gridDim.x) {
        const int4 tk = task[t];
        double v[1] = {0.0};
        if (sc[tk.x].active) {
            const double alpha = sc[tk.x].alpha;
            const size_t slot = (size_t)(sc[tk.x].iter % M) * n;
            for (long i = tk.y + threadIdx.x; i < tk.z; i += blockDim.x) {
                const double pi = p[i], qi = q[i];
                x[i] += alpha * pi;
                const double ri = r[i] - alpha * qi;
                r[i] = ri;
                v[0] += ri * ri;
                ph[slot + i] = pi;
                qh[slot + i] = qi;
            }
        } else {
            for (long i = tk.y + threadIdx.x; i < tk.z; i += blockDim.x) v[0] += r[i] * r[i];
        }
        seg_block_sums<1>(v, part + t);
    }
}

// Per system (one warp each): its tasks' partials summed in task order, then the scalars of MODE.  In
// SEG_RR the kernel also sets the loop condition: some system still active.
template <int MODE, int M>
__global__ void __launch_bounds__(1024) seg_finish_kernel(int S, const int* __restrict__ tbeg,
                                                          const double* __restrict__ part, SegScalars* sc,
                                                          cudaGraphConditionalHandle hd, int set_cond, int* act) {
    pdl_wait();
    constexpr int W = (MODE == SEG_DOT) ? M + 1 : 1;
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int mine = 0;
    for (int s = w; s < S; s += nw) {
        double tot[W];
#pragma unroll
        for (int k = 0; k < W; k++) {
            double x = 0.0;
            for (int t = tbeg[s] + lane; t < tbeg[s + 1]; t += 32) x += part[(size_t)t * W + k];
            tot[k] = warp_sum(x);
        }
        if (lane != 0) continue;
        SegScalars& c = sc[s];
        if constexpr (MODE == SEG_DOT) {
            if (c.active) {
                const int k = c.iter;
                const int nprev = min(k - c.base, M);
                c.s_old = c.s;
                c.s = tot[0];
#pragma unroll
                for (int j = 1; j <= M; j++) {
                    c.tj[j - 1] = tot[j];
                    c.cj[j - 1] = (j <= nprev) ? tot[j] / c.pqh[(k - j + M * kFcgMax) % M] : 0.0;
                }
            }
        } else if constexpr (MODE == SEG_PQ) {
            if (c.active) {
                c.pq = tot[0];
                c.alpha = c.s / tot[0];
            }
        } else if constexpr (MODE == SEG_RR) {
            c.rr = tot[0];
            if (c.active) {
                c.pqh[c.iter % M] = c.pq;
                c.iter += 1;
                const double rel = sqrt(c.rr) / c.r0;
                if (!isfinite(rel)) {
                    c.status = LINA_GPU_EBREAKDOWN;
                    c.active = 0;
                } else if (rel <= c.tol || c.iter >= c.maxit) {
                    c.active = 0;
                }
            }
            mine |= c.active;
            act[s] = c.active;
        } else if constexpr (MODE == SEG_NORM_B) {
            c.r0 = sqrt(tot[0]);
            c.rr = tot[0];
            c.iter = 0;
            c.base = 0;
            c.status = 0;
            c.s = 0.0;
            c.active = (c.r0 > 0.0 && isfinite(c.r0) && c.maxit > 0) ? 1 : 0;
            mine |= c.active;
            act[s] = c.active;
        } else {
            c.tnorm2 = tot[0];
        }
    }
    if constexpr (MODE == SEG_RR || MODE == SEG_NORM_B) {
        if (mine) atomicOr(&any, 1);
        __syncthreads();
        if (threadIdx.x == 0 && set_cond) cudaGraphSetConditional(hd, any ? 1u : 0u);
    }
}

// combined hierarchy: level l of system i is its level l - (D - d_i), or a copy of its coarsest level
struct SegLevelMap {
    std::vector<std::vector<int>> off;  // off[l][i]: first row of system i on combined level l (size S+1)
};

lina::Csr identity_csr(int n) {
    lina::Csr I;
    I.n = n;
    I.ncols = n;
    I.ptr.resize(n + 1);
    I.col.resize(n);
    I.val.assign(n, 1.0);
    for (int i = 0; i <= n; i++) I.ptr[i] = i;
    for (int i = 0; i < n; i++) I.col[i] = i;
    return I;
}

// block-diagonal concatenation of parts (each with its row and column offsets)
lina::Csr concat_csr(const std::vector<const lina::Csr*>& parts, const std::vector<int>& roff,
                     const std::vector<int>& coff, int ncols) {
    lina::Csr C;
    long nnz = 0;
    for (const lina::Csr* p : parts) nnz += p->nnz();
    C.n = roff.back();
    C.ncols = ncols;
    C.ptr.assign(C.n + 1, 0);
    C.col.resize(nnz);
    C.val.resize(nnz);
    long at = 0;
    for (size_t i = 0; i < parts.size(); i++) {
        const lina::Csr& P = *parts[i];
        for (int r = 0; r < P.n; r++) C.ptr[roff[i] + r + 1] = (int)(at + P.ptr[r + 1]);
        for (long k = 0; k < P.nnz(); k++) {
            C.col[at + k] = P.col[k] + coff[i];
            C.val[at + k] = P.val[k];
        }
        at += P.nnz();
    }
    return C;
}

int combine_hierarchies(const std::vector<lina_gpu_amg*>& sys, lina::HostHierarchy& C, SegLevelMap& map) {
    const int S = (int)sys.size();
    int D = 0;
    for (auto* h : sys) D = std::max(D, h->depth);
    auto lev = [&](int i, int l) { return l - (D - sys[i]->depth); };  // system i's own level (< 0: padded)
    C.params = sys[0]->host.params;
    C.params.depth = D;
    C.lv.assign(D, lina::HostLevel());
    map.off.assign(D, std::vector<int>(S + 1, 0));
    for (int l = 0; l < D; l++)
        for (int i = 0; i < S; i++) {
            const int li = std::max(lev(i, l), 0);
            map.off[l][i + 1] = map.off[l][i] + sys[i]->host.lv[li].A.n;
        }
    for (int l = 0; l < D; l++) {
        std::vector<const lina::Csr*> parts(S);
        for (int i = 0; i < S; i++) parts[i] = &sys[i]->host.lv[std::max(lev(i, l), 0)].A;
        lina::HostLevel& L = C.lv[l];
        L.A = concat_csr(parts, map.off[l], map.off[l], map.off[l][S]);
        L.dof_level.assign(L.A.n, 0);
        for (int i = 0; i < S; i++) {
            const lina::HostLevel& Hi = sys[i]->host.lv[std::max(lev(i, l), 0)];
            if ((int)Hi.dof_level.size() == Hi.A.n)
                std::copy(Hi.dof_level.begin(), Hi.dof_level.end(), L.dof_level.begin() + map.off[l][i]);
        }
        if (l == 0) continue;
        L.labels.assign(L.A.n, lina::kCoarse);
        std::vector<lina::Csr> ids;
        ids.reserve(S);
        std::vector<const lina::Csr*> ps(S), rs(S);
        for (int i = 0; i < S; i++) {
            const int li = lev(i, l);
            if (li >= 1) {
                const lina::HostLevel& Hi = sys[i]->host.lv[li];
                ps[i] = &Hi.P;
                rs[i] = &Hi.R;
                if ((int)Hi.labels.size() == Hi.A.n)
                    std::copy(Hi.labels.begin(), Hi.labels.end(), L.labels.begin() + map.off[l][i]);
            } else {
                ids.push_back(identity_csr(sys[i]->host.lv[0].A.n));
                ps[i] = rs[i] = &ids.back();
            }
        }
        L.P = concat_csr(ps, map.off[l], map.off[l - 1], map.off[l - 1][S]);
        L.R = concat_csr(rs, map.off[l - 1], map.off[l], map.off[l][S]);
        L.coarse_size = map.off[l - 1][S];
    }
    // the coarsest level: each system's own dense block
    lina::CoarseSolver& cs = C.coarse;
    cs = lina::CoarseSolver();
    cs.n = map.off[0][S];
    cs.in_block.assign(cs.n, 0);
    cs.diag_inv.assign(cs.n, 0.0);
    cs.blocks.assign(1, 0);
    cs.inv_offsets.assign(1, 0);
    for (int i = 0; i < S; i++) {
        const lina::CoarseSolver& ci = sys[i]->host.coarse;
        const int o = map.off[0][i];
        for (int r : ci.block_rows) cs.block_rows.push_back(r + o);
        for (int r = 0; r < ci.n; r++) {
            cs.in_block[o + r] = ci.in_block[r];
            cs.diag_inv[o + r] = ci.diag_inv[r];
        }
        cs.inv.insert(cs.inv.end(), ci.inv.begin(), ci.inv.end());
        cs.blocks.push_back((int)cs.block_rows.size());
        cs.inv_offsets.push_back((long)cs.inv.size());
        cs.block_inverted.push_back(ci.inverted ? 1 : 0);
    }
    cs.inverted = true;
    return 0;
}

}  // namespace

struct lina_gpu_segbatch {
    std::vector<lina_gpu_amg*> sys;
    lina_gpu_amg* comb = nullptr;   // the combined hierarchy (owned)
    std::vector<int> off;           // finest rows of system i: [off[i], off[i+1])
    int ntask = 0;
    int4* task = nullptr;           // (system, first row, end row, 0)
    int* tbeg = nullptr;            // tasks of system i: [tbeg[i], tbeg[i+1])
    double* part = nullptr;         // ntask x (M + 1)
    SegScalars* sc = nullptr;       // device, one per system
    int* act = nullptr;             // device, one per system: still iterating (the row masks read it)
    SegScalars* sc_host = nullptr;  // pinned
    int m = 1;                      // FCG history
    cudaGraphExec_t exec = nullptr;
    long k_iter = 0;                // kernels per iteration
    ~lina_gpu_segbatch() {
        if (comb && comb->stream) cudaStreamSynchronize(comb->stream);
        if (exec) cudaGraphExecDestroy(exec);
        if (sc_host) cudaFreeHost(sc_host);
        delete comb;  // frees task, tbeg, part, sc (allocated through it)
    }
};

namespace {

template <int M>
void seg_issue_iteration(lina_gpu_segbatch* B, cudaGraphConditionalHandle hd, int set_cond) {
    lina_gpu_amg* h = B->comb;
    const long n = h->lv[h->depth - 1].n;
    const int S = (int)B->sys.size();
    const bool mixed = (h->opt.precision == LINA_PREC_MIXED);
    const int gt = std::min(B->ntask, kGridCap);
    cudaStream_t st = h->stream;
    h->precondition(h->kr, h->kz, false);
    if (mixed)
        go(seg_fcg_dot_kernel<float, M>, gt, st, B->ntask, (const int4*)B->task, n, (const double*)h->kr,
           (const float*)h->kz32, (const double*)h->kqh, (const SegScalars*)B->sc, B->part);
    else
        go(seg_fcg_dot_kernel<double, M>, gt, st, B->ntask, (const int4*)B->task, n, (const double*)h->kr,
           (const double*)h->kz, (const double*)h->kqh, (const SegScalars*)B->sc, B->part);
    launch(seg_finish_kernel<SEG_DOT, M>, dim3(1), dim3(1024), 0, st, S, (const int*)B->tbeg,
           (const double*)B->part, B->sc, hd, 0, B->act);
    if (mixed)
        go(seg_fcg_update_p_kernel<float, M>, gt, st, B->ntask, (const int4*)B->task, n, (const float*)h->kz32,
           (const double*)h->kph, h->kp, (const SegScalars*)B->sc);
    else
        go(seg_fcg_update_p_kernel<double, M>, gt, st, B->ntask, (const int4*)B->task, n, (const double*)h->kz,
           (const double*)h->kph, h->kp, (const SegScalars*)B->sc);
    h->csr<double, M_SPMV>(h->krylov_matrix(), h->kp, h->kq);
    go(seg_dot_kernel, gt, st, B->ntask, (const int4*)B->task, (const double*)h->kp, (const double*)h->kq, B->part);
    launch(seg_finish_kernel<SEG_PQ, M>, dim3(1), dim3(1024), 0, st, S, (const int*)B->tbeg, (const double*)B->part,
           B->sc, hd, 0, B->act);
    go(seg_update_xr_kernel<M>, gt, st, B->ntask, (const int4*)B->task, n, h->kx, h->kr, (const double*)h->kp,
       (const double*)h->kq, h->kph, h->kqh, (const SegScalars*)B->sc, B->part);
    launch(seg_finish_kernel<SEG_RR, M>, dim3(1), dim3(1024), 0, st, S, (const int*)B->tbeg, (const double*)B->part,
           B->sc, hd, set_cond, B->act);
}

void seg_issue(lina_gpu_segbatch* B, cudaGraphConditionalHandle hd, int set_cond) {
    switch (B->m) {
        case 1: seg_issue_iteration<1>(B, hd, set_cond); break;
        case 2: seg_issue_iteration<2>(B, hd, set_cond); break;
        case 3: seg_issue_iteration<3>(B, hd, set_cond); break;
        case 4: seg_issue_iteration<4>(B, hd, set_cond); break;
        case 5: seg_issue_iteration<5>(B, hd, set_cond); break;
        case 6: seg_issue_iteration<6>(B, hd, set_cond); break;
        case 7: seg_issue_iteration<7>(B, hd, set_cond); break;
        default: seg_issue_iteration<8>(B, hd, set_cond); break;
    }
}

int seg_build_graph(lina_gpu_segbatch* B) {
    lina_gpu_amg* h = B->comb;
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle hd;
    cudaError_t e = cudaGraphConditionalHandleCreate(&hd, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams cp = {};
    cudaGraphNode_t node;
    if (e == cudaSuccess) {
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = hd;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
    }
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(h->stream, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        set_err("segmented batch graph: %s", cudaGetErrorString(e));
        return LINA_GPU_ECUDA;
    }
    const unsigned long long before = g_launches;
    h->mask_rows = true;
    seg_issue(B, hd, 1);
    h->mask_rows = false;
    B->k_iter = (long)(g_launches - before);
    g_launches = before;
    cudaGraph_t body = nullptr;
    e = cudaStreamEndCapture(h->stream, &body);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&B->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        B->exec = nullptr;
        set_err("segmented batch graph: %s", cudaGetErrorString(e));
        return LINA_GPU_ECUDA;
    }
    return 0;
}

// the per-system norms of v (SEG_NORM_B: ||b|| and the start of the loop; SEG_NORM_T: ||b - A x||^2)
template <int MODE>
void seg_norms(lina_gpu_segbatch* B, const double* v) {
    lina_gpu_amg* h = B->comb;
    const int gt = std::min(B->ntask, kGridCap);
    go(seg_dot_kernel, gt, h->stream, B->ntask, (const int4*)B->task, v, v, B->part);
    launch(seg_finish_kernel<MODE, 1>, dim3(1), dim3(1024), 0, h->stream, (int)B->sys.size(), (const int*)B->tbeg,
           (const double*)B->part, B->sc, (cudaGraphConditionalHandle)0, 0, B->act);
}

}  // namespace

extern "C" {

int lina_gpu_segbatch_create(int count, lina_gpu_amg* const* systems, lina_gpu_segbatch** out) {
    if (count < 1 || !systems || !out) {
        set_err("lina_gpu_segbatch_create: invalid argument");
        return LINA_GPU_EINVAL;
    }
    *out = nullptr;
    const lina_gpu_amg* s0 = systems[0];
    for (int i = 0; i < count; i++) {
        const lina_gpu_amg* h = systems[i];
        if (!h || h->host_only || h->has_signs || h->depth < 1 || h->opt.smoother != s0->opt.smoother ||
            h->opt.omega != s0->opt.omega || h->opt.precision != s0->opt.precision ||
            h->opt.smoothing_iterations != s0->opt.smoothing_iterations ||
            (h->opt.coarsening == LINA_AGGRESSIVE) != (s0->opt.coarsening == LINA_AGGRESSIVE) ||
            h->opt.aggr_smoothing_iterations != s0->opt.aggr_smoothing_iterations) {
            set_err("lina_gpu_segbatch_create: system %d is not a device hierarchy with the first system's smoother, "
                    "precision and sweeps (or its rows were sign-flipped)", i);
            return LINA_GPU_EINVAL;
        }
    }
    lina_gpu_segbatch* B = new lina_gpu_segbatch();
    B->sys.assign(systems, systems + count);
    lina_gpu_amg* c = new lina_gpu_amg();
    B->comb = c;
    SegLevelMap map;
    combine_hierarchies(B->sys, c->host, map);
    c->opt = s0->opt;
    c->depth = (int)c->host.lv.size();
    c->opt.depth = c->depth;
    c->seg_max_rows.assign(c->depth, 0);
    for (int l = 0; l < c->depth; l++)
        for (int i = 0; i < count; i++)
            c->seg_max_rows[l] = std::max<long>(c->seg_max_rows[l], map.off[l][i + 1] - map.off[l][i]);
    c->seg_off = map.off;
    c->autotune = true;  // the concatenated levels' layouts are measured
    c->fcg_m = s0->fcg_m;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete B;
        set_err("cudaStreamCreate failed");
        return LINA_GPU_ECUDA;
    }
    int rc = upload_hierarchy(c);
    if (!rc) {
        B->m = std::max(c->history(), 1);
        if (B->m >= 2) rc = c->ensure_history();
        if (!rc && B->m == 1) {  // a ring of one slot for the two-term recurrence
            const size_t n = (size_t)c->lv[c->depth - 1].n;
            if (!(rc = c->alloc(&c->kph, n))) rc = c->alloc(&c->kqh, n);
        }
    }
    if (rc) {
        delete B;
        return rc;
    }
    B->off = map.off[c->depth - 1];
    std::vector<int4> tasks;
    std::vector<int> tbeg(count + 1, 0);
    for (int i = 0; i < count; i++) {
        for (int r = B->off[i]; r < B->off[i + 1]; r += kSegChunk)
            tasks.push_back(make_int4(i, r, std::min(r + kSegChunk, B->off[i + 1]), 0));
        tbeg[i + 1] = (int)tasks.size();
    }
    B->ntask = (int)tasks.size();
    if ((rc = c->upload(&B->task, tasks.data(), tasks.size())) || (rc = c->upload(&B->tbeg, tbeg.data(), tbeg.size())) ||
        (rc = c->alloc(&B->part, (size_t)B->ntask * (kFcgMax + 1))) || (rc = c->alloc(&B->sc, count)) ||
        (rc = c->alloc(&B->act, count))) {
        delete B;
        return rc;
    }
    // the system of every row of every level, for the row masks of the iteration
    for (int l = 0; l < c->depth; l++) {
        std::vector<int> seg(map.off[l][count]);
        for (int i = 0; i < count; i++)
            for (int r = map.off[l][i]; r < map.off[l][i + 1]; r++) seg[r] = i;
        int* d = nullptr;
        if ((rc = c->upload(&d, seg.data(), seg.size()))) {
            delete B;
            return rc;
        }
        DLevel& L = c->lv[l];
        L.A.rowseg = L.Acol.rowseg = L.P.rowseg = d;
        L.A.act = L.Acol.act = L.P.act = L.R.act = B->act;
        if (l + 1 < c->depth) c->lv[l + 1].R.rowseg = d;  // R of level l+1 has level l's rows
    }
    CK(cudaMemsetAsync(B->act, 0, count * sizeof(int), c->stream));
    if (cudaMallocHost((void**)&B->sc_host, count * sizeof(SegScalars)) != cudaSuccess) {
        delete B;
        set_err("cudaMallocHost failed");
        return LINA_GPU_ECUDA;
    }
    CK(cudaStreamSynchronize(c->stream));
    if ((rc = seg_build_graph(B))) {
        delete B;
        return rc;
    }
    *out = B;
    return 0;
}

int lina_gpu_segbatch_solve(lina_gpu_segbatch* B, const double* const* b, double* const* x, double tol, int max_iter,
                            int flags, lina_gpu_solve_info* infos) {
    if (!B || !b || !x || max_iter < 1 || !(tol > 0.0)) {
        set_err("lina_gpu_segbatch_solve: invalid argument");
        return LINA_GPU_EINVAL;
    }
    const int S = (int)B->sys.size();
    for (int i = 0; i < S; i++)
        if (!b[i] || !x[i]) {
            set_err("lina_gpu_segbatch_solve: missing vector of system %d", i);
            return LINA_GPU_EINVAL;
        }
    lina_gpu_amg* h = B->comb;
    cudaStream_t st = h->stream;
    const bool dev = (flags & LINA_PCG_DEVICE_PTRS) != 0;
    const long n = h->lv[h->depth - 1].n;
    for (int i = 0; i < S; i++)
        CK(cudaMemcpyAsync(h->kb + B->off[i], b[i], (size_t)(B->off[i + 1] - B->off[i]) * sizeof(double),
                           dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    // x = 0, r = b, per-system ||b||, tolerance and limit
    CK(cudaMemsetAsync(h->kx, 0, n * sizeof(double), st));
    CK(cudaMemcpyAsync(h->kr, h->kb, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemsetAsync(B->sc, 0, S * sizeof(SegScalars), st));
    for (int i = 0; i < S; i++) {
        B->sc_host[i] = SegScalars{};
        B->sc_host[i].tol = tol;
        B->sc_host[i].maxit = max_iter;
    }
    CK(cudaMemcpyAsync(B->sc, B->sc_host, S * sizeof(SegScalars), cudaMemcpyHostToDevice, st));
    seg_norms<SEG_NORM_B>(B, h->kb);
    std::vector<int> restarts(S, 0);
    int rounds = 0;
    const bool host_loop = (flags & LINA_PCG_HOST_LOOP) != 0;
    for (;;) {
        if (host_loop) {  // iteration by iteration from the host (kernels visible to a profiler)
            for (int it = 0; it < max_iter; it++) {
                h->mask_rows = true;
                seg_issue(B, (cudaGraphConditionalHandle)0, 0);
                h->mask_rows = false;
                CK(cudaMemcpyAsync(B->sc_host, B->sc, S * sizeof(SegScalars), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                bool any = false;
                for (int i = 0; i < S; i++) any = any || B->sc_host[i].active;
                if (!any) break;
            }
        } else {
            CK(cudaGraphLaunch(B->exec, st));
        }
        // the true residual of every system
        h->csr<double, M_RESID>(h->krylov_matrix(), h->kx, h->kt, h->kb);
        seg_norms<SEG_NORM_T>(B, h->kt);
        CK(cudaMemcpyAsync(B->sc_host, B->sc, S * sizeof(SegScalars), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        long its = 0;
        for (int i = 0; i < S; i++) its = std::max<long>(its, B->sc_host[i].iter - B->sc_host[i].base);
        g_launches += (unsigned long long)(its * B->k_iter + 3);
        // systems whose recursive residual met the rule but whose true residual does not: restart
        // from the true residual (a new recurrence; FCG history cleared) while iterations remain
        bool again = false;
        for (int i = 0; i < S; i++) {
            SegScalars& c = B->sc_host[i];
            const double trel = c.r0 > 0.0 ? std::sqrt(c.tnorm2) / c.r0 : 0.0;
            if (c.status == 0 && c.r0 > 0.0 && trel > tol && c.iter < max_iter && rounds < 8) {
                CK(cudaMemcpyAsync(h->kr + B->off[i], h->kt + B->off[i],
                                   (size_t)(B->off[i + 1] - B->off[i]) * sizeof(double), cudaMemcpyDeviceToDevice,
                                   st));
                c.active = 1;
                c.base = c.iter;
                restarts[i]++;
                again = true;
            }
        }
        if (!again) break;
        rounds++;
        CK(cudaMemcpyAsync(B->sc, B->sc_host, S * sizeof(SegScalars), cudaMemcpyHostToDevice, st));
        std::vector<int> act_host(S);
        for (int i = 0; i < S; i++) act_host[i] = B->sc_host[i].active;
        CK(cudaMemcpyAsync(B->act, act_host.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));  // act_host goes out of scope
    }
    for (int i = 0; i < S; i++)
        CK(cudaMemcpyAsync(x[i], h->kx + B->off[i], (size_t)(B->off[i + 1] - B->off[i]) * sizeof(double),
                           dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int rc = 0;
    for (int i = 0; i < S; i++) {
        const SegScalars& c = B->sc_host[i];
        lina_gpu_solve_info inf{};
        inf.iterations = c.iter;
        inf.rel_residual = c.r0 > 0.0 ? std::sqrt(c.rr) / c.r0 : 0.0;
        inf.true_rel_residual = c.r0 > 0.0 ? std::sqrt(c.tnorm2) / c.r0 : 0.0;
        inf.status = c.status;
        if (!inf.status && inf.true_rel_residual > tol) inf.status = LINA_GPU_ENOCONV;
        inf.restarts = restarts[i];
        if (infos) infos[i] = inf;
        if (inf.status && !rc) rc = inf.status == LINA_GPU_ENOCONV ? LINA_GPU_ENOCONV : inf.status;
    }
    return rc;
}

int lina_gpu_segbatch_levels(const lina_gpu_segbatch* B, int* depth, long* rows, long* entries) {
    if (!B || !depth) return LINA_GPU_EINVAL;
    *depth = B->comb->depth;
    for (int l = 0; l < B->comb->depth; l++) {
        if (rows) rows[l] = B->comb->lv[l].n;
        if (entries) entries[l] = B->comb->lv[l].A.nnz;
    }
    return 0;
}

int lina_gpu_segbatch_hierarchy(lina_gpu_segbatch* B, lina_gpu_amg** out) {
    if (!B || !out) return LINA_GPU_EINVAL;
    *out = B->comb;
    return 0;
}

int lina_gpu_segbatch_destroy(lina_gpu_segbatch* B) {
    delete B;
    return 0;
}

}  // extern "C"
