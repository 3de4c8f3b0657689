// gpu_ilu.cu - ILU(0) factorisation and application on the GPU.
//
// The factors are the reference's (incomplete_LU_factorization,
// LinA/linear_algebra.c:1952-1982, with row_times_row :1795): on A's pattern,
// row by row, L_ij = a_ij - sum_{k<j} L_ik U_kj for j <= i and
// U_ij = (a_ij - sum_{k<i} L_ik U_kj) / L_ii for j > i (U has a unit
// diagonal; the sums run over k in ascending order).  Applying the
// preconditioner is the forward solve L y = r and the backward solve U z = y
// (L_triang_invert / U_triang_invert, :2008-2043).
//
// Both the factorisation and the solves are row-by-row recurrences: a row
// needs the finished rows it couples to (smaller indices for the factorisation
// and the forward solve, larger ones for the backward solve).  Rows are ordered
// by level (one more than the highest level among the rows they need) and a
// fixed pool of warps takes them in that order, 32 rows (one per lane) per
// ticket from a counter; a row waits only for the rows it needs.  A warp takes
// a ticket only after all smaller tickets were taken by running warps, and it
// finishes its rows before it takes the next, so every row waited for is being
// worked on: the passes cannot deadlock, whatever the launch order of blocks.
// In the solves a row waits on the solution entries themselves: the pass first
// fills x with a NaN pattern that arithmetic never produces (a result with that
// pattern is stored as the canonical NaN), and an entry is final once it no
// longer holds the pattern (aligned 32- and 64-bit stores are single-copy
// atomic).  The factorisation publishes a row's values and then a flag holding
// the pass number.  The waits are bounded: a wait that runs out sets an error
// code that the host reads, and the pass ends instead of spinning on.  Products
// and sums of the factorisation are rounded one at a time in the reference's
// order, so the factors are bit-identical to the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "bulk_copy.cuh"
#include "gpu_ops.h"
#include "lina_gpu.h"

namespace {

constexpr int kT = 256;      // threads of the elementwise kernels
constexpr int kPool = 128;   // threads of a block of the worker pool
// a wait gives up after kWaitNs of device time (or kWaitPolls polls, whichever comes first); the
// longest legitimate wait is the time the pool needs for the rows taken before a row, far below it
constexpr unsigned long long kWaitNs = 2000000000ull;
constexpr long kWaitPolls = 1L << 26;
constexpr unsigned kMaxSleepNs = 256;
constexpr int kGroup = 8;  // solution entries a row of a triangular solve loads at once

cudaStream_t st() { return (cudaStream_t)lina::dev::stream(); }

__device__ __forceinline__ unsigned long long device_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// the next 32 rows of the order for this warp (the same value in every lane)
__device__ __forceinline__ int take_chunk(unsigned* ticket) {
    unsigned c = 0;
    if ((threadIdx.x & 31) == 0) c = atomicAdd(ticket, 1u);
    return (int)__shfl_sync(0xffffffffu, c, 0);
}

// bounded wait with back-off; `ready` polls the awaited value.  False (and *err = 1) when the wait
// runs out or a pass failed elsewhere
template <typename Ready>
__device__ __forceinline__ bool wait_for(Ready ready, int* err, unsigned long long limit_ns = kWaitNs) {
    if (ready()) return true;
    const unsigned long long t0 = device_ns();
    long polls = 0;
    unsigned ns = 32;
    while (!ready()) {
        if (++polls > kWaitPolls || *(volatile int*)err || device_ns() - t0 > limit_ns) {
            atomicCAS(err, 0, 1);
            return false;
        }
        __nanosleep(ns);
        ns = ns < kMaxSleepNs ? 2 * ns : kMaxSleepNs;
    }
    return true;
}

template <typename T>
struct Word;
template <>
struct Word<float> {
    using U = unsigned;
    static constexpr U kPending = 0xffffffffu;   // a NaN arithmetic does not produce
    static constexpr U kNaN = 0x7fc00000u;
};
template <>
struct Word<double> {
    using U = unsigned long long;
    static constexpr U kPending = 0xffffffffffffffffull;
    static constexpr U kNaN = 0x7ff8000000000000ull;
};

template <typename T>
__device__ __forceinline__ typename Word<T>::U bits(T v) {
    typename Word<T>::U u;
    memcpy(&u, &v, sizeof(T));
    return u;
}
template <typename T>
__device__ __forceinline__ T from_bits(typename Word<T>::U u) {
    T v;
    memcpy(&v, &u, sizeof(T));
    return v;
}

// x_i = (b_i - sum_{p in [beg_i, end_i)} val_p x_{col_p}) * dinv_i (dinv null: unit diagonal), rows in
// `order`; x holds the pending pattern on entry
template <typename TV, typename TX>
__global__ void __launch_bounds__(kPool) sptrsv_kernel(int n, const int* __restrict__ order,
                                                       const int* __restrict__ beg, const int* __restrict__ end,
                                                       const int* __restrict__ col, const TV* __restrict__ val,
                                                       const TX* __restrict__ dinv, const TX* __restrict__ b, TX* x,
                                                       unsigned* ticket, int* err) {
    using U = typename Word<TX>::U;
    volatile U* xw = reinterpret_cast<volatile U*>(x);
    const int nchunks = (n + 31) >> 5;
    for (int c = take_chunk(ticket); c < nchunks; c = take_chunk(ticket)) {
        const int t = c * 32 + (threadIdx.x & 31);
        if (t < n) {
            const int i = order[t];
            const int p1 = end[i];
            TX s = b[i];
            bool ok = true;
            // the entries of a group are loaded together, and while some are pending all of those are
            // read again together, so a row whose needed rows finish at about the same time waits one
            // round trip, not one per entry; then the products are subtracted in column order
            for (int p = beg[i]; p < p1; p += kGroup) {
                int k[kGroup];
                U u[kGroup];
#pragma unroll
                for (int q = 0; q < kGroup; q++) k[q] = p + q < p1 ? col[p + q] : -1;
#pragma unroll
                for (int q = 0; q < kGroup; q++) u[q] = k[q] >= 0 ? xw[k[q]] : U(0);
                ok = ok && wait_for(
                               [&] {
                                   bool all = true;
#pragma unroll
                                   for (int q = 0; q < kGroup; q++)
                                       if (k[q] >= 0 && u[q] == Word<TX>::kPending) {
                                           u[q] = xw[k[q]];
                                           all = all && u[q] != Word<TX>::kPending;
                                       }
                                   return all;
                               },
                               err);
#pragma unroll
                for (int q = 0; q < kGroup; q++)
                    if (k[q] >= 0) s -= TX(val[p + q]) * from_bits<TX>(u[q]);
            }
            TX r = dinv ? s * dinv[i] : s;
            U ur = bits(r);
            if (ur == Word<TX>::kPending || !ok) ur = Word<TX>::kNaN;
            xw[i] = ur;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- one-block level-synchronous solves
// A triangular solve whose rows are listed level by level (positions), run by one block: the rows of
// a level in parallel, a __syncthreads between levels.  The solution entries of the last
// kWinLevels + 1 levels stay in a shared-memory ring (slot = position mod ring size), so a row reads
// the rows it needs from shared memory; entries of older levels are read back from the
// position-major solution in global memory, which the block itself wrote.  Each level's rows (first
// entry, b, 1/L_ii) and entries (encoded source, value) lie contiguously in position-major arrays,
// each level's slice 16-byte aligned, and one thread copies them into shared memory S - 1 levels
// ahead with bulk (TMA) copies completing on a per-stage barrier: a level then costs
// shared-memory reads, a few products and a block barrier.  The stages are kept small (a row's
// entries end where the next row's begin) to fit many.  Products are subtracted in the factor's
// entry order, so the results equal sptrsv_kernel's.
constexpr int kWinLevels = 3;               // levels back whose entries the ring holds
constexpr int kWinThreads = 1024;
constexpr int kWinSmemMax = 220 * 1024;
constexpr int kWinMaxStages = 6;

__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

struct WinLayout {  // byte offsets inside one stage
    int head, dinv, b, enc, val, bytes;
};
__host__ __device__ inline WinLayout win_layout(int max_rows, int max_ent, int tx, int tv, bool dinv) {
    WinLayout L;
    L.head = 0;
    L.dinv = align16(L.head + 4 * max_rows);
    L.b = align16(L.dinv + (dinv ? tx * max_rows : 0));
    L.enc = align16(L.b + tx * max_rows);
    L.val = align16(L.enc + 4 * max_ent);
    L.bytes = align16(L.val + tv * max_ent);
    return L;
}

template <typename TV, typename TX>
struct WinArgs {
    int nlev, ringmask, max_rows, max_ent;
    const int4* bounds;  // level -> (first position, rows, first packed entry, entries); starts are
                         // multiples of 4, so every level's slice of every array is 16-byte aligned
    const int* head;     // position -> first packed entry
    const int* enc;      // packed entry -> ring slot, or -(position + 1) of an older row
    const TV* val;       // packed entry -> factor value
    const TX* dinv;      // position -> 1 / L_ii (null: unit diagonal)
    const TX* bpos;      // position -> right-hand side
    TX* xpos;            // position -> solution
    int* err;            // set when a wait for a copy runs out
};

// the bulk copies' barriers (one per stage) wait with this file's error word, code 4
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int* err) {
    return bulk::mbar_wait(bar, parity, err, 4, kWaitNs);
}

// the issuing thread: bulk-copy level l's slices (16-byte aligned, sizes multiples of 16) into stage l % S;
// the stage's barrier completes when all bytes have landed
template <typename TV, typename TX, int S>
__device__ __forceinline__ void win_issue(const WinArgs<TV, TX>& a, unsigned char* stages, uint64_t* bars,
                                          const WinLayout& L, int l, int4 bd) {
    unsigned char* st = stages + (l % S) * L.bytes;
    uint64_t* bar = bars + (l % S);
    const int pr = (bd.y + 3) & ~3, pe = (bd.w + 3) & ~3;  // padded rows and entries
    const unsigned nb_head = 4u * pr, nb_dinv = a.dinv ? (unsigned)sizeof(TX) * pr : 0u,
                   nb_b = (unsigned)sizeof(TX) * pr, nb_enc = 4u * pe, nb_val = (unsigned)sizeof(TV) * pe;
    // the stage was last read through ordinary loads; order those before the copies' writes
    bulk::fence_proxy_async();
    bulk::mbar_expect_tx(bar, nb_head + nb_dinv + nb_b + nb_enc + nb_val);
    auto put = [&](unsigned char* dst, const void* src, unsigned bytes) {
        if (bytes) bulk::copy(dst, src, bytes, bar);
    };
    put(st + L.head, a.head + bd.x, nb_head);
    if (a.dinv) put(st + L.dinv, a.dinv + bd.x, nb_dinv);
    put(st + L.b, a.bpos + bd.x, nb_b);
    put(st + L.enc, a.enc + bd.z, nb_enc);
    put(st + L.val, a.val + bd.z, nb_val);
}

template <typename TV, typename TX, int S, bool RING_ONLY>
__global__ void __launch_bounds__(kWinThreads, 1) sptrsv_window_kernel(const WinArgs<TV, TX> a) {
    extern __shared__ __align__(16) unsigned char win_smem[];
    const int tid = threadIdx.x, T = blockDim.x;
    uint64_t* bars = reinterpret_cast<uint64_t*>(win_smem);
    TX* ring = reinterpret_cast<TX*>(win_smem + align16(8 * S));
    unsigned char* stages = win_smem + align16(8 * S) + align16((a.ringmask + 1) * (int)sizeof(TX));
    const WinLayout L = win_layout(a.max_rows, a.max_ent, sizeof(TX), sizeof(TV), a.dinv != nullptr);
    // the copies are issued by the block's last thread: rows go to the lowest threads first, so on
    // levels narrower than the block its warp has no row and the issue costs the level nothing
    const int issuer = T - 1;
    if (tid == issuer) {
        for (int k = 0; k < S; k++) bulk::mbar_init(bars + k);
        bulk::fence_mbar_init();
        for (int l = 0; l < S - 1 && l < a.nlev; l++) win_issue<TV, TX, S>(a, stages, bars, L, l, __ldg(a.bounds + l));
    }
    __syncthreads();
    // bounds of the level being solved and of the next one to copy, loaded one level ahead
    int4 cur = __ldg(a.bounds);
    int4 nb = S - 1 < a.nlev ? __ldg(a.bounds + S - 1) : make_int4(0, 0, 0, 0);
    for (int l = 0; l < a.nlev; l++) {
        // the stage of level l + S - 1 was read in level l - 1, which every thread has finished
        if (tid == issuer && l + S - 1 < a.nlev) win_issue<TV, TX, S>(a, stages, bars, L, l + S - 1, nb);
        const int4 nb2 = l + S < a.nlev ? __ldg(a.bounds + l + S) : make_int4(0, 0, 0, 0);
        const int4 next = l + 1 < a.nlev ? __ldg(a.bounds + l + 1) : make_int4(0, 0, 0, 0);
        mbar_wait(bars + (l % S), (unsigned)((l / S) & 1), a.err);
        const unsigned char* st = stages + (l % S) * L.bytes;
        const int* head = reinterpret_cast<const int*>(st + L.head);
        const TX* dv = reinterpret_cast<const TX*>(st + L.dinv);
        const TX* bv = reinterpret_cast<const TX*>(st + L.b);
        const int* enc = reinterpret_cast<const int*>(st + L.enc);
        const TV* val = reinterpret_cast<const TV*>(st + L.val);
        const int t0 = cur.x, nr = cur.y, q0 = cur.z, qe = cur.z + cur.w;
        for (int r = tid; r < nr; r += T) {
            const int k0 = head[r] - q0, k1 = (r + 1 < nr ? head[r + 1] : qe) - q0;
            TX s = bv[r];
            for (int k = k0; k < k1; k++) {
                const int e = enc[k];
                const TX v = (RING_ONLY || e >= 0) ? ring[e] : __ldcg(a.xpos + (-e - 1));
                s -= TX(val[k]) * v;
            }
            const TX res = a.dinv ? s * dv[r] : s;
            ring[(t0 + r) & a.ringmask] = res;
            a.xpos[t0 + r] = res;
        }
        __syncthreads();
        cur = next;
        nb = nb2;
    }
    // after a failed wait no copy of this block may still be landing when it exits: wait (bounded,
    // not cut short by the error) for the last stages' copies
    if (tid == issuer && *(volatile int*)a.err)
        for (int l = a.nlev > S ? a.nlev - S : 0; l < a.nlev; l++)
            bulk::mbar_drain(bars + (l % S), (unsigned)((l / S) & 1), kWaitNs);
}

// bpos[t] = b[row[t]] (0 on padding positions): the right-hand side in position order
template <typename TX>
__global__ void gather_pos_kernel(int n, const int* __restrict__ row, const TX* __restrict__ b, TX* __restrict__ bpos) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        bpos[t] = row[t] >= 0 ? b[row[t]] : TX(0);
}

// x[row[t]] = xpos[t]: the solution from position order (padding positions skipped)
template <typename TX>
__global__ void scatter_pos_kernel(int n, const int* __restrict__ row, const TX* __restrict__ xpos, TX* __restrict__ x) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        if (row[t] >= 0) x[row[t]] = xpos[t];
}


// packed copies of the factor values (entry order of the window) and of 1/L_ii (position order)
__global__ void pack_values_kernel(long ne, const int* __restrict__ perm, const double* __restrict__ v64,
                                   const float* __restrict__ v32, double* __restrict__ w64, float* __restrict__ w32) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < ne; q += (long)gridDim.x * blockDim.x) {
        const int p = perm[q];  // -1: padding
        w64[q] = p >= 0 ? v64[p] : 0.0;
        w32[q] = p >= 0 ? v32[p] : 0.0f;
    }
}

// one thread waits, through wait_for, for a flag that nothing sets: the wait must run out after
// limit_ns, record the failure in *err and return (the failure path of every bounded wait above)
__global__ void wait_probe_kernel(const int* flag, unsigned long long limit_ns, int* err,
                                  unsigned long long* waited_ns) {
    const unsigned long long t0 = device_ns();
    wait_for([&] { return *(volatile const int*)flag != 0; }, err, limit_ns);
    *waited_ns = device_ns() - t0;
}

__device__ __forceinline__ void publish_row(int* flag, int i, int epoch) {
    __threadfence();
    *(volatile int*)(flag + i) = epoch;
}

// position of column j in [lo, e) of the sorted column array (row k's upper part: U_kj)
__device__ __forceinline__ bool find_upper(const int* col, int lo, int e, int j, int* pos) {
    int hi = e - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int c = col[mid];
        if (c == j) {
            *pos = mid;
            return true;
        }
        if (c < j)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return false;
}

// wait until the rows col[q] (q in [q0, q1), the entries left of the diagonal) show this pass,
// polling up to eight flags together
__device__ __forceinline__ bool wait_rows(const int* __restrict__ col, int q0, int q1, const int* flag, int epoch,
                                          int* err) {
    for (int q = q0; q < q1; q += 8) {
        int k[8];
        bool done[8];
#pragma unroll
        for (int t = 0; t < 8; t++) {
            k[t] = q + t < q1 ? __ldg(col + q + t) : -1;
            done[t] = k[t] < 0;
        }
        const bool ok = wait_for(
            [&] {
                bool all = true;
#pragma unroll
                for (int t = 0; t < 8; t++)
                    if (!done[t]) {
                        done[t] = *(volatile const int*)(flag + k[t]) == epoch;
                        all = all && done[t];
                    }
                return all;
            },
            err);
        if (!ok) return false;
    }
    return true;
}

// One row of the factorisation with the row and the upper parts of the rows it needs staged in
// local arrays (rows of up to kRowMax entries, up to kLowMax of them left of the diagonal, needed
// rows with up to kUMax entries right of theirs; false, with nothing waited for or written,
// otherwise).  Everything that does not depend on other rows' factors (the pattern, A's values)
// is loaded before the wait, the needed rows' factors in one batch after it.  The needed rows
// k < i are taken in ascending order: L_ik is final when k is reached (its sum has every term from
// rows before k), and the products L_ik U_kj are added to the sums of the entries j > k that row
// k's upper part shares with row i.  Every sum thus gets its terms in ascending k, as in
// row_times_row, rounded one at a time.
constexpr int kRowMax = 32, kLowMax = 8, kUMax = 16;

__device__ __forceinline__ int ilu0_row_staged(int i, int r0, int r1, const int* __restrict__ ptr,
                                               const int* __restrict__ col, const double* __restrict__ a,
                                               const int* __restrict__ ustart, double* f, const int* flag,
                                               int epoch, int* err) {
    const int len = r1 - r0;
    if (len > kRowMax) return 0;
    int cj[kRowMax];
    int nlow = 0;
    for (int p = 0; p < len; p++) {
        cj[p] = __ldg(col + r0 + p);
        if (cj[p] < i) nlow = p + 1;
    }
    if (nlow > kLowMax) return 0;
    int u0[kLowMax], nu[kLowMax];
    for (int q = 0; q < nlow; q++) {
        u0[q] = __ldg(ustart + cj[q]);
        nu[q] = __ldg(ptr + cj[q] + 1) - u0[q];
        if (nu[q] > kUMax) return 0;
    }
    double av[kRowMax], sum[kRowMax];
    for (int p = 0; p < len; p++) {
        av[p] = __ldg(a + r0 + p);
        sum[p] = 0.0;
    }
    int uc[kLowMax][kUMax];
    for (int q = 0; q < nlow; q++)
        for (int t = 0; t < nu[q]; t++) uc[q][t] = __ldg(col + u0[q] + t);
    if (!wait_rows(col, r0, r0 + nlow, flag, epoch, err)) return -1;
    __threadfence();
    double uv[kLowMax][kUMax];
    for (int q = 0; q < nlow; q++)
        for (int t = 0; t < nu[q]; t++) uv[q][t] = __ldcg(f + u0[q] + t);
    for (int q = 0; q < nlow; q++) {
        const double L = __dsub_rn(av[q], sum[q]);
        f[r0 + q] = L;
        int pp = q + 1;
        for (int t = 0; t < nu[q] && pp < len; t++) {
            const int j = uc[q][t];
            while (pp < len && cj[pp] < j) pp++;
            if (pp < len && cj[pp] == j) sum[pp] = __dadd_rn(sum[pp], __dmul_rn(L, uv[q][t]));
        }
    }
    double d = 0.0;  // L_ii (0 where the pattern has no diagonal)
    for (int p = nlow; p < len; p++) {
        const double v = __dsub_rn(av[p], sum[p]);
        if (cj[p] == i) {
            f[r0 + p] = v;
            d = v;
        } else {
            if (d == 0.0) {
                atomicExch(err, 2);
                break;
            }
            f[r0 + p] = __ddiv_rn(v, d);
        }
    }
    return 1;
}

// ILU(0) of A (CSR, sorted columns) into f on A's pattern, rows in forward level order; ustart_k is
// the first entry of row k right of the diagonal; *err = 2 on a zero pivot (the reference's failure),
// 1 if a wait ran out
__device__ __forceinline__ void ilu0_row(int i, const int* __restrict__ ptr, const int* __restrict__ col,
                                         const double* __restrict__ a, const int* __restrict__ diagpos,
                                         const int* __restrict__ ustart, double* f, int* flag, int epoch, int* err) {
    const int r0 = ptr[i], r1 = ptr[i + 1];
    const int staged = ilu0_row_staged(i, r0, r1, ptr, col, a, ustart, f, flag, epoch, err);
    if (staged == 0) {
        int nlow = 0;
        while (r0 + nlow < r1 && col[r0 + nlow] < i) nlow++;
        if (wait_rows(col, r0, r0 + nlow, flag, epoch, err)) {
            __threadfence();
            const int di = diagpos[i];
            for (int p = r0; p < r1; p++) {
                const int j = col[p];
                const int jmax = (j <= i) ? j - 1 : i - 1;
                double s = 0.0;
                for (int q = r0; q < r1 && col[q] <= jmax; q++) {
                    const int k = col[q];
                    int pos;
                    if (find_upper(col, __ldg(ustart + k), ptr[k + 1], j, &pos))
                        s = __dadd_rn(s, __dmul_rn(__ldcg(f + q), __ldcg(f + pos)));
                }
                const double v = __dsub_rn(a[p], s);
                if (j <= i) {
                    f[p] = v;
                } else {
                    const double d = di >= 0 ? __ldcg(f + di) : 0.0;
                    if (d == 0.0) {
                        atomicExch(err, 2);
                        break;
                    }
                    f[p] = __ddiv_rn(v, d);
                }
            }
        }
    }
    publish_row(flag, i, epoch);
}

__global__ void __launch_bounds__(kPool) ilu0_kernel(int n, const int* __restrict__ order, const int* __restrict__ ptr,
                                                     const int* __restrict__ col, const double* __restrict__ a,
                                                     const int* __restrict__ diagpos, const int* __restrict__ ustart,
                                                     double* f, int* flag, int epoch, unsigned* ticket, int* err) {
    const int nchunks = (n + 31) >> 5;
    for (int c = take_chunk(ticket); c < nchunks; c = take_chunk(ticket)) {
        const int t = c * 32 + (threadIdx.x & 31);
        if (t < n) ilu0_row(order[t], ptr, col, a, diagpos, ustart, f, flag, epoch, err);
        __syncwarp();
    }
}

// 1/L_ii from the factor array (0 where the pattern has no diagonal: a division by zero follows,
// as in the reference's triangular solve)
__global__ void diag_inverse_kernel(int n, const int* __restrict__ diagpos, const double* __restrict__ f,
                                    double* dinv64, float* dinv32) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double d = diagpos[i] >= 0 ? f[diagpos[i]] : 0.0;
        const double v = 1.0 / d;
        dinv64[i] = v;
        dinv32[i] = float(v);
    }
}

template <typename TA, typename TB>
__global__ void cvt_kernel(long n, const TA* __restrict__ a, TB* __restrict__ b) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = TB(a[i]);
}

template <typename T>
__global__ void fill_kernel(long n, T v, T* __restrict__ a) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) a[i] = v;
}

// one triangular factor as row segments [beg_i, end_i) of shared column and value arrays
struct Factor {
    int nlev = 0;
    int *order = nullptr, *beg = nullptr, *end = nullptr, *col = nullptr;
    double *val64 = nullptr, *dinv64 = nullptr;
    float *val32 = nullptr, *dinv32 = nullptr;  // dinv null: unit diagonal
    // the one-block level-synchronous solve (s32 / s64 = 0: the row pool in that precision)
    struct Win {
        int s32 = 0, s64 = 0;  // cp.async stages
        int ringmask = 0, max_rows = 0, max_ent = 0;
        long ne = 0;      // packed entries (padded)
        bool ring_only = true;  // every needed row lies within the ring's levels
        int npos = 0;     // positions (padded)
        size_t smem32 = 0, smem64 = 0;
        int *bounds = nullptr, *head = nullptr, *row = nullptr, *enc = nullptr, *vperm = nullptr;
        double *val64 = nullptr, *dinv64 = nullptr;
        float *val32 = nullptr, *dinv32 = nullptr;
    } win;
};

struct Mem {
    std::vector<void*> p;
    template <typename T>
    T* get(size_t count) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        p.push_back(q);
        return (T*)q;
    }
    template <typename T>
    T* up(const T* h, size_t count) {
        T* d = get<T>(count);
        if (d && count && cudaMemcpy(d, h, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
        return d;
    }
    template <typename T>
    T* up(const std::vector<T>& h) {
        return up(h.data(), h.size());
    }
    ~Mem() {
        for (void* q : p) cudaFree(q);
    }
};

// level order of rows: lower = rows need smaller indices (entries [beg_i, end_i) columns), else larger
int level_order(int n, const std::vector<int>& beg, const std::vector<int>& end, const int* col, bool lower,
                std::vector<int>& order, std::vector<int>* lev_out = nullptr, std::vector<int>* lp_out = nullptr) {
    std::vector<int> lev(n, 0);
    int nlev = 0;
    for (int t = 0; t < n; t++) {
        const int i = lower ? t : n - 1 - t;
        int l = 0;
        for (int k = beg[i]; k < end[i]; k++) l = std::max(l, lev[col[k]] + 1);
        lev[i] = l;
        nlev = std::max(nlev, l + 1);
    }
    std::vector<int> lp(nlev + 1, 0);
    for (int i = 0; i < n; i++) lp[lev[i] + 1]++;
    for (int l = 0; l < nlev; l++) lp[l + 1] += lp[l];
    order.assign(n, 0);
    for (int i = 0; i < n; i++) order[lp[lev[i]]++] = i;
    if (lp_out) {  // level starts (lp was advanced to the ends by the fill)
        lp_out->assign(nlev + 1, 0);
        for (int l = 0; l < nlev; l++) (*lp_out)[l + 1] = lp[l];
    }
    if (lev_out) lev_out->swap(lev);
    return nlev;
}

std::string g_ilu_err;

// blocks of the worker pool: enough warps to keep the widest levels busy, few enough that the
// waiting warps do not crowd the memory system (LINA_ILU_POOL_BLOCKS_PER_SM, default 2 per SM: on
// 1M- and 2M-row mesh matrices 1 and 2 blocks per SM were fastest, 4 about 10 % and 8 about 70 % slower)
int pool_blocks(int n) {
    static int per_grid = 0;
    if (per_grid == 0) {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            sms = 1;
        int per_sm = 2;
        if (const char* e = getenv("LINA_ILU_POOL_BLOCKS_PER_SM")) per_sm = std::max(1, std::min(16, atoi(e)));
        per_grid = sms * per_sm;
    }
    return std::max(1, std::min(per_grid, (n + kPool - 1) / kPool));
}

}  // namespace

struct lina_gpu_ilu {
    int n = 0;
    Factor L, U;
    Mem mem;
    double* t64 = nullptr;
    float *r32 = nullptr, *t32 = nullptr, *z32 = nullptr;
    int* err = nullptr;
    unsigned* ticket = nullptr;  // the pool's row counter, reset before every pass
    double *bpos64 = nullptr, *xpos64 = nullptr;  // position-major work of the one-block solves
    float *bpos32 = nullptr, *xpos32 = nullptr;
    int npos = 0;                                  // their length
    int* flag = nullptr;         // rows finished by the factorisation
    double* fval = nullptr;      // factor values on A's pattern (factorised on the device), else null
    int epoch = 0;               // factorisation passes (row flags hold the current one)
    int *aptr = nullptr, *acol = nullptr, *adiag = nullptr;  // A's pattern (device factorisation)
    double* aval = nullptr;                                  // A's values
    long fnnz = 0;
};

namespace {

bool alloc_work(lina_gpu_ilu* h) {
    const int n = h->n;
    h->t64 = h->mem.get<double>(n);
    h->r32 = h->mem.get<float>(n);
    h->t32 = h->mem.get<float>(n);
    h->z32 = h->mem.get<float>(n);
    h->err = h->mem.get<int>(1);
    h->ticket = h->mem.get<unsigned>(1);
    return h->t64 && h->r32 && h->t32 && h->z32 && h->err && h->ticket &&
           cudaMemset(h->err, 0, sizeof(int)) == cudaSuccess;
}

// The one-block solve's position-major arrays for a factor: levels from level_order (lev, lp), row
// i's needed entries [beg_i, end_i) of the column array col (in the order they are subtracted).
// Disabled (no stages) where its shared memory would not fit.
template <typename TV, typename TX>
size_t win_smem(int ring, int max_rows, int max_ent, bool dinv, int stages) {
    return (size_t)align16(8 * stages) + align16(ring * (int)sizeof(TX)) +
           (size_t)stages * win_layout(max_rows, max_ent, sizeof(TX), sizeof(TV), dinv).bytes;
}

// host side of a factor's window layout (plan_window) and its upload (upload_window); the plan
// needs no device, so the plans of L and U can be made at the same time
struct WinPlan {
    Factor::Win w;
    std::vector<int> head, row, enc, vperm, bounds;
};

void plan_window(WinPlan& pl, int n, const std::vector<int>& order, const std::vector<int>& lev,
                 const std::vector<int>& lp, const std::vector<int>& beg, const std::vector<int>& end, const int* col,
                 bool has_dinv) {
    Factor::Win& w = pl.w;
    w = Factor::Win();
    const int nlev = (int)lp.size() - 1;
    if (nlev <= 0) return;
    // padded positions and entries: every level starts at a multiple of 4 in both
    std::vector<int> P(nlev + 1, 0), Q(nlev + 1, 0), ecount(nlev, 0);
    long ptot = 0, qtot = 0;
    for (int l = 0; l < nlev; l++) {
        long e = 0;
        for (int t = lp[l]; t < lp[l + 1]; t++) e += end[order[t]] - beg[order[t]];
        ecount[l] = (int)e;
        P[l] = (int)ptot;
        Q[l] = (int)qtot;
        ptot += (lp[l + 1] - lp[l] + 3) & ~3;
        qtot += (e + 3) & ~3;
        if (ptot > INT32_MAX / 4 || qtot > INT32_MAX / 4) return;  // too large: the row pool
    }
    P[nlev] = (int)ptot;
    Q[nlev] = (int)qtot;
    std::vector<int> ppos(n);
    for (int l = 0; l < nlev; l++)
        for (int t = lp[l]; t < lp[l + 1]; t++) ppos[order[t]] = P[l] + (t - lp[l]);
    int maxwin = 0, max_rows = 0, max_ent = 0;
    for (int l = 0; l < nlev; l++) {
        maxwin = std::max(maxwin, P[l + 1] - P[std::max(0, l - kWinLevels)]);
        max_rows = std::max(max_rows, P[l + 1] - P[l]);
        max_ent = std::max(max_ent, Q[l + 1] - Q[l]);
    }
    int ring = 1;
    while (ring < maxwin) ring *= 2;
    for (int S = kWinMaxStages; S >= 2 && w.s32 == 0; S--)
        if (win_smem<float, float>(ring, max_rows, max_ent, has_dinv, S) <= (size_t)kWinSmemMax) w.s32 = S;
    for (int S = kWinMaxStages; S >= 2 && w.s64 == 0; S--)
        if (win_smem<double, double>(ring, max_rows, max_ent, has_dinv, S) <= (size_t)kWinSmemMax) w.s64 = S;
    if (w.s32 == 0 && w.s64 == 0) return;
    pl.head.assign(ptot, 0);
    pl.row.assign(ptot, -1);
    pl.enc.assign(qtot, 0);
    pl.vperm.assign(qtot, -1);
    pl.bounds.assign(4 * (size_t)nlev, 0);
    int* head = pl.head.data();
    int* row = pl.row.data();
    int* enc = pl.enc.data();
    int* vperm = pl.vperm.data();
    int* bounds = pl.bounds.data();
    int older = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : older)
    for (int l = 0; l < nlev; l++) {
        int q = Q[l];
        for (int t = lp[l]; t < lp[l + 1]; t++) {
            const int i = order[t], pp = P[l] + (t - lp[l]);
            row[pp] = i;
            head[pp] = q;
            for (int p = beg[i]; p < end[i]; p++, q++) {
                const int j = col[p];
                vperm[q] = p;
                enc[q] = lev[i] - lev[j] <= kWinLevels ? (ppos[j] & (ring - 1)) : -(ppos[j] + 1);
                if (enc[q] < 0) older = 1;
            }
        }
        bounds[4 * (size_t)l] = P[l];
        bounds[4 * (size_t)l + 1] = lp[l + 1] - lp[l];
        bounds[4 * (size_t)l + 2] = Q[l];
        bounds[4 * (size_t)l + 3] = ecount[l];
    }
    w.ring_only = older == 0;
    w.ringmask = ring - 1;
    w.max_rows = max_rows;
    w.max_ent = max_ent;
    w.ne = qtot;
    w.npos = (int)ptot;
    if (w.s32) w.smem32 = win_smem<float, float>(ring, max_rows, max_ent, has_dinv, w.s32);
    if (w.s64) w.smem64 = win_smem<double, double>(ring, max_rows, max_ent, has_dinv, w.s64);
}

// the plan's arrays on the device; a factor without a plan (levels too wide or too large) keeps
// the row pool
bool upload_window(lina_gpu_ilu* h, Factor& f, const WinPlan& pl, bool has_dinv) {
    Factor::Win& w = f.win;
    w = pl.w;
    if (!w.s32 && !w.s64) return true;
    Mem& m = h->mem;
    w.bounds = m.up(pl.bounds);
    w.head = m.up(pl.head);
    w.row = m.up(pl.row);
    w.enc = m.up(pl.enc);
    w.vperm = m.up(pl.vperm);
    w.val64 = m.get<double>(w.ne);
    w.val32 = m.get<float>(w.ne);
    bool ok = w.bounds && w.head && w.row && w.enc && w.vperm && w.val64 && w.val32;
    if (has_dinv) {
        w.dinv64 = m.get<double>(w.npos);
        w.dinv32 = m.get<float>(w.npos);
        ok = ok && w.dinv64 && w.dinv32;
    }
    if (ok && h->npos < w.npos) {  // position-major work vectors, shared by both factors
        h->bpos64 = m.get<double>(w.npos);
        h->xpos64 = m.get<double>(w.npos);
        h->bpos32 = m.get<float>(w.npos);
        h->xpos32 = m.get<float>(w.npos);
        ok = h->bpos64 && h->xpos64 && h->bpos32 && h->xpos32;
        h->npos = w.npos;
    }
    if (!ok) {
        w = Factor::Win();
        return false;
    }
    return true;
}

bool build_window(lina_gpu_ilu* h, Factor& f, int n, const std::vector<int>& order, const std::vector<int>& lev,
                  const std::vector<int>& lp, const std::vector<int>& beg, const std::vector<int>& end,
                  const int* col, bool has_dinv) {
    WinPlan pl;
    plan_window(pl, n, order, lev, lp, beg, end, col, has_dinv);
    return upload_window(h, f, pl, has_dinv);
}

// the window's packed copies of a factor's values and inverse diagonal (after every factorisation)
void pack_window(Factor& f, int n) {
    Factor::Win& w = f.win;
    if (!w.s32 && !w.s64) return;
    pack_values_kernel<<<std::min<long>(4096, (w.ne + kT - 1) / kT), kT, 0, st()>>>(w.ne, w.vperm, f.val64, f.val32,
                                                                                   w.val64, w.val32);
    if (w.dinv64) {
        const int g = std::min(4096, (w.npos + kT - 1) / kT);
        gather_pos_kernel<double><<<g, kT, 0, st()>>>(w.npos, w.row, f.dinv64, w.dinv64);
        gather_pos_kernel<float><<<g, kT, 0, st()>>>(w.npos, w.row, f.dinv32, w.dinv32);
    }
}

// a factor given as CSR with its diagonal (lower: L with diagonal; upper: U, diagonal 1 skipped)
bool build_factor(lina_gpu_ilu* h, Factor& f, int n, const int* p, const int* c, const double* v, bool lower,
                  std::string& err) {
    std::vector<int> ptr(n + 1, 0), col;
    std::vector<double> val, dinv(n, 0.0);
    col.reserve(p[n]);
    val.reserve(p[n]);
    for (int i = 0; i < n; i++) {
        double d = 0.0;
        if (p[i + 1] < p[i]) {
            err = "row pointers of a factor decrease";
            return false;
        }
        for (int k = p[i]; k < p[i + 1]; k++) {
            if (c[k] < 0 || c[k] >= n) {
                err = "column index of a factor outside the matrix";
                return false;
            }
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
    std::vector<int> beg(ptr.begin(), ptr.end() - 1), end(ptr.begin() + 1, ptr.end()), order;
    std::vector<int> lev, lp;
    f.nlev = level_order(n, beg, end, col.data(), lower, order, &lev, &lp);
    std::vector<float> val32(val.begin(), val.end()), dinv32(dinv.begin(), dinv.end());
    int* dptr = h->mem.up(ptr);
    f.order = h->mem.up(order);
    f.col = h->mem.up(col);
    f.val64 = h->mem.up(val);
    f.val32 = h->mem.up(val32);
    // an upper factor with the reference's unit diagonal needs no scaling
    bool unit = !lower;
    for (int i = 0; unit && i < n; i++) unit = (dinv[i] == 1.0);
    if (!unit) {
        f.dinv64 = h->mem.up(dinv);
        f.dinv32 = h->mem.up(dinv32);
    }
    if (!dptr || !f.order || !f.col || !f.val64 || !f.val32 || (!unit && (!f.dinv64 || !f.dinv32))) {
        err = "device allocation for the ILU factors failed";
        return false;
    }
    f.beg = dptr;
    f.end = dptr + 1;
    if (!build_window(h, f, n, order, lev, lp, beg, end, col.data(), !unit)) {
        err = "device allocation for the ILU factors failed";
        return false;
    }
    pack_window(f, n);
    return true;
}

int read_err(lina_gpu_ilu* h) {
    int e = 0;
    if (cudaMemcpyAsync(&e, h->err, sizeof(int), cudaMemcpyDeviceToHost, st()) != cudaSuccess ||
        cudaStreamSynchronize(st()) != cudaSuccess)
        return -1;
    return e;
}

// ILU(0) of the handle's A (pattern and values on the device) into fval, the inverse diagonal and
// the FP32 copy of the factors; each factorisation is a new pass of the row flags
int factorise(lina_gpu_ilu* h) {
    const int n = h->n;
    const long nnz = h->fnnz;
    h->epoch++;
    cudaMemsetAsync(h->ticket, 0, sizeof(unsigned), st());
    ilu0_kernel<<<pool_blocks(n), kPool, 0, st()>>>(n, h->L.order, h->aptr, h->acol, h->aval, h->adiag, h->U.beg,
                                                    h->fval, h->flag, h->epoch, h->ticket, h->err);
    diag_inverse_kernel<<<std::min(4096, (n + kT - 1) / kT), kT, 0, st()>>>(n, h->adiag, h->fval, h->L.dinv64,
                                                                             h->L.dinv32);
    cvt_kernel<double, float><<<std::min<long>(4096, (nnz + kT - 1) / kT), kT, 0, st()>>>(nnz, h->fval, h->L.val32);
    pack_window(h->L, n);
    pack_window(h->U, n);
    const int e = (cudaGetLastError() == cudaSuccess) ? read_err(h) : -1;
    if (e != 0) {
        lina::dev::set_error(e == 2 ? "ILU: zero pivot (incomplete_LU_factorization fails)"
                                    : "ILU: device factorisation failed or a wait ran out");
        if (e > 0) cudaMemset(h->err, 0, sizeof(int));
        return e == 2 ? LINA_GPU_ESETUP : LINA_GPU_ECUDA;
    }
    return 0;
}

template <typename TV, typename TX, int S, bool RING_ONLY>
void launch_window_t(const WinArgs<TV, TX>& a, size_t smem) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(sptrsv_window_kernel<TV, TX, S, RING_ONLY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kWinSmemMax);
        attr = true;
    }
    sptrsv_window_kernel<TV, TX, S, RING_ONLY><<<1, kWinThreads, smem, st()>>>(a);
}

template <typename TV, typename TX, int S>
void launch_window(lina_gpu_ilu* h, const Factor& f, const WinArgs<TV, TX>& a, size_t smem) {
    (void)h;
    if (f.win.ring_only)
        launch_window_t<TV, TX, S, true>(a, smem);
    else
        launch_window_t<TV, TX, S, false>(a, smem);
}

template <typename TV, typename TX>
void solve(lina_gpu_ilu* h, const Factor& f, const TV* val, const TX* dinv, const TX* b, TX* x) {
    const int n = h->n;
    const Factor::Win& w = f.win;
    const int stages = sizeof(TX) == 8 ? w.s64 : w.s32;
    if (stages) {
        WinArgs<TV, TX> a;
        a.nlev = f.nlev;
        a.ringmask = w.ringmask;
        a.max_rows = w.max_rows;
        a.max_ent = w.max_ent;
        a.bounds = reinterpret_cast<const int4*>(w.bounds);
        a.head = w.head;
        a.enc = w.enc;
        TX* bpos;
        if constexpr (sizeof(TX) == 8) {
            a.val = (const TV*)w.val64;
            a.dinv = dinv ? (const TX*)w.dinv64 : nullptr;
            bpos = (TX*)h->bpos64;
            a.xpos = (TX*)h->xpos64;
        } else {
            a.val = (const TV*)w.val32;
            a.dinv = dinv ? (const TX*)w.dinv32 : nullptr;
            bpos = (TX*)h->bpos32;
            a.xpos = (TX*)h->xpos32;
        }
        a.bpos = bpos;
        a.err = h->err;
        const int g = std::min(4096, (w.npos + kT - 1) / kT);
        gather_pos_kernel<TX><<<g, kT, 0, st()>>>(w.npos, w.row, b, bpos);
        const size_t smem = sizeof(TX) == 8 ? w.smem64 : w.smem32;
        switch (stages) {
            case 6: launch_window<TV, TX, 6>(h, f, a, smem); break;
            case 5: launch_window<TV, TX, 5>(h, f, a, smem); break;
            case 4: launch_window<TV, TX, 4>(h, f, a, smem); break;
            case 3: launch_window<TV, TX, 3>(h, f, a, smem); break;
            default: launch_window<TV, TX, 2>(h, f, a, smem); break;
        }
        scatter_pos_kernel<TX><<<g, kT, 0, st()>>>(w.npos, w.row, a.xpos, x);
        return;
    }
    cudaMemsetAsync(x, 0xff, (size_t)n * sizeof(TX), st());  // every entry pending
    cudaMemsetAsync(h->ticket, 0, sizeof(unsigned), st());
    sptrsv_kernel<TV, TX><<<pool_blocks(n), kPool, 0, st()>>>(n, f.order, f.beg, f.end, f.col, val, dinv, b, x,
                                                              h->ticket, h->err);
}

}  // namespace

extern "C" {

int lina_gpu_ilu_create(int n, const int* Lptr, const int* Lcol, const double* Lval, const int* Uptr,
                        const int* Ucol, const double* Uval, lina_gpu_ilu** out) {
    if (!out || n <= 0 || !Lptr || !Lcol || !Lval || !Uptr || !Ucol || !Uval) return LINA_GPU_EINVAL;
    *out = nullptr;
    lina_gpu_ilu* h = new lina_gpu_ilu();
    h->n = n;
    std::string err;
    if (!lina::dev::ready() || !build_factor(h, h->L, n, Lptr, Lcol, Lval, true, err) ||
        !build_factor(h, h->U, n, Uptr, Ucol, Uval, false, err) || !alloc_work(h)) {
        g_ilu_err = err.empty() ? "device allocation failed" : err;
        lina::dev::set_error(("ILU: " + g_ilu_err).c_str());
        delete h;
        return LINA_GPU_EINVAL;
    }
    *out = h;
    return 0;
}

// ILU(0) of A factorised on the device (bit-identical to the reference's incomplete_LU_factorization).
// LINA_ILU_TIMING set: seconds per set-up phase on stderr (diagnostics).
int lina_gpu_ilu_create_from_matrix(int n, const int* rowptr, const int* col, const double* val,
                                    lina_gpu_ilu** out) {
    const bool timing = getenv("LINA_ILU_TIMING") != nullptr;
    auto t_prev = std::chrono::steady_clock::now();
    auto lap = [&](const char* what) {
        if (!timing) return;
        cudaStreamSynchronize(st());
        const auto now = std::chrono::steady_clock::now();
        fprintf(stderr, "ILU set-up %s %.1f ms\n", what, std::chrono::duration<double>(now - t_prev).count() * 1e3);
        t_prev = now;
    };
    if (!out || n <= 0 || !rowptr || !col || !val || rowptr[0] != 0) return LINA_GPU_EINVAL;
    *out = nullptr;
    const long nnz = rowptr[n];
    std::vector<int> diag(n, -1), lbeg(n), lend(n), ubeg(n), uend(n);
    for (int i = 0; i < n; i++)
        if (rowptr[i + 1] < rowptr[i]) return LINA_GPU_EINVAL;
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int i = 0; i < n; i++) {
        int split = rowptr[i + 1];
        for (int p = rowptr[i]; p < rowptr[i + 1]; p++) {
            if (col[p] < 0 || col[p] >= n || (p > rowptr[i] && col[p] <= col[p - 1])) bad = 1;
            if (col[p] == i) diag[i] = p;
            if (col[p] > i && split == rowptr[i + 1]) split = p;
        }
        lbeg[i] = rowptr[i];
        lend[i] = diag[i] >= 0 ? diag[i] : split;  // strictly lower entries
        ubeg[i] = split;
        uend[i] = rowptr[i + 1];
    }
    if (bad) {
        lina::dev::set_error("ILU: columns must be sorted, distinct and inside the matrix");
        return LINA_GPU_EINVAL;
    }
    lina_gpu_ilu* h = new lina_gpu_ilu();
    h->n = n;
    h->fnnz = nnz;
    std::vector<int> lorder, uorder, llev, ulev, llp, ulp;
    lap("pattern checks and splits");
    // the level schedules and window plans of L and U are independent: U's on a second thread
    WinPlan lplan, uplan;
    std::thread upper([&] {
        h->U.nlev = level_order(n, ubeg, uend, col, false, uorder, &ulev, &ulp);
        plan_window(uplan, n, uorder, ulev, ulp, ubeg, uend, col, false);
    });
    h->L.nlev = level_order(n, lbeg, lend, col, true, lorder, &llev, &llp);
    plan_window(lplan, n, lorder, llev, llp, lbeg, lend, col, true);
    upper.join();
    lap("level schedules and window plans");
    Mem& m = h->mem;
    int *dptr = nullptr, *dcol = nullptr, *ddiag = nullptr;
    double* dval = nullptr;
    bool ok = lina::dev::ready() && alloc_work(h);
    if (ok) {
        dptr = m.up(rowptr, (size_t)n + 1);
        dcol = m.up(col, (size_t)nnz);
        ddiag = m.up(diag);
        dval = m.up(val, (size_t)nnz);
        h->fval = m.get<double>(nnz);
        h->L.order = m.up(lorder);
        h->U.order = m.up(uorder);
        h->L.beg = m.up(lbeg);
        h->L.end = m.up(lend);
        h->U.beg = m.up(ubeg);
        h->U.end = m.up(uend);
        h->L.dinv64 = m.get<double>(n);
        h->L.dinv32 = m.get<float>(n);
        h->L.val32 = m.get<float>(nnz);
        ok = dptr && dcol && ddiag && dval && h->fval && h->L.order && h->U.order && h->L.beg && h->L.end &&
             h->U.beg && h->U.end && h->L.dinv64 && h->L.dinv32 && h->L.val32;
    }
    if (!ok) {
        lina::dev::set_error("ILU: device allocation failed");
        delete h;
        return LINA_GPU_ECUDA;
    }
    lap("uploads");
    h->L.col = h->U.col = dcol;
    h->L.val64 = h->U.val64 = h->fval;
    h->U.val32 = h->L.val32;
    if (!upload_window(h, h->L, lplan, true) || !upload_window(h, h->U, uplan, false)) {
        lina::dev::set_error("ILU: device allocation failed");
        delete h;
        return LINA_GPU_ECUDA;
    }
    h->flag = m.get<int>(n);
    h->aptr = dptr;
    h->acol = dcol;
    h->adiag = ddiag;
    h->aval = dval;
    if (!h->flag || cudaMemsetAsync(h->flag, 0, (size_t)n * sizeof(int), st()) != cudaSuccess) {
        lina::dev::set_error("ILU: device allocation failed");
        delete h;
        return LINA_GPU_ECUDA;
    }
    lap("window uploads");
    const int rc = factorise(h);
    if (rc) {
        delete h;
        return rc;
    }
    lap("factorisation");
    *out = h;
    return 0;
}

// new values of A on the pattern the handle was created with (val[nnz], host or, with
// LINA_PCG_DEVICE_PTRS, device pointer): the factors are recomputed on the device, the level
// schedules and the pattern are kept
int lina_gpu_ilu_refactor(lina_gpu_ilu* h, const double* val, int flags) {
    if (!h || !val || !h->fval) {
        lina::dev::set_error("lina_gpu_ilu_refactor: not a handle factorised on the device");
        return LINA_GPU_EINVAL;
    }
    const cudaMemcpyKind kind = (flags & LINA_PCG_DEVICE_PTRS) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (h->fnnz && cudaMemcpyAsync(h->aval, val, (size_t)h->fnnz * sizeof(double), kind, st()) != cudaSuccess) {
        lina::dev::set_error("lina_gpu_ilu_refactor: copy of the values failed");
        return LINA_GPU_ECUDA;
    }
    return factorise(h);
}

// The failure path of the bounded device waits, made to happen: a kernel waits up to limit_us
// microseconds (at most one second) for a flag nothing sets.  Returns LINA_GPU_ECUDA with the
// error text set, as the solves do when a wait runs out, and the time the wait took in
// *waited_us; the device stays usable.
int lina_gpu_wait_probe(int limit_us, double* waited_us) {
    if (limit_us <= 0 || limit_us > 1000000) return LINA_GPU_EINVAL;
    Mem m;
    int* flag = m.get<int>(1);
    int* err = m.get<int>(1);
    unsigned long long* waited = m.get<unsigned long long>(1);
    if (!flag || !err || !waited || cudaMemsetAsync(flag, 0, sizeof(int), st()) != cudaSuccess ||
        cudaMemsetAsync(err, 0, sizeof(int), st()) != cudaSuccess)
        return LINA_GPU_ECUDA;
    wait_probe_kernel<<<1, 1, 0, st()>>>(flag, 1000ull * (unsigned long long)limit_us, err, waited);
    int e = 0;
    unsigned long long ns = 0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, st()) != cudaSuccess ||
        cudaMemcpyAsync(&ns, waited, sizeof(ns), cudaMemcpyDeviceToHost, st()) != cudaSuccess ||
        cudaStreamSynchronize(st()) != cudaSuccess)
        return LINA_GPU_ECUDA;
    if (waited_us) *waited_us = ns / 1000.0;
    if (e != 0) {
        lina::dev::set_error("a device wait ran out (no row ever published the awaited value)");
        return LINA_GPU_ECUDA;
    }
    return 0;
}

int lina_gpu_ilu_destroy(lina_gpu_ilu* h) {
    if (h) cudaStreamSynchronize(st());
    delete h;
    return 0;
}

int lina_gpu_ilu_levels(const lina_gpu_ilu* h, int* nlev_L, int* nlev_U) {
    if (!h) return LINA_GPU_EINVAL;
    if (nlev_L) *nlev_L = h->L.nlev;
    if (nlev_U) *nlev_U = h->U.nlev;
    return 0;
}

int lina_gpu_ilu_factor_values(const lina_gpu_ilu* h, double* val) {
    if (!h || !val || !h->fval) {
        lina::dev::set_error("lina_gpu_ilu_factor_values: not a handle factorised on the device");
        return LINA_GPU_EINVAL;
    }
    if (h->fnnz && cudaMemcpy(val, h->fval, h->fnnz * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
        return LINA_GPU_ECUDA;
    return 0;
}

// z = U^-1 L^-1 r on device vectors (FP64); precision LINA_PREC_MIXED runs both solves in FP32.
// The work is issued on the stream of the device vector toolkit and completes before return.
int lina_gpu_ilu_apply(lina_gpu_ilu* h, int precision, const double* r_dev, double* z_dev) {
    if (!h || !r_dev || !z_dev) return LINA_GPU_EINVAL;
    const int n = h->n;
    const int g = (int)std::min<long>(2048, (n + kT - 1) / kT);
    if (precision == LINA_PREC_MIXED) {
        cvt_kernel<double, float><<<g, kT, 0, st()>>>(n, r_dev, h->r32);
        solve<float, float>(h, h->L, h->L.val32, h->L.dinv32, h->r32, h->t32);
        solve<float, float>(h, h->U, h->U.val32, h->U.dinv32, h->t32, h->z32);
        cvt_kernel<float, double><<<g, kT, 0, st()>>>(n, h->z32, z_dev);
    } else {
        solve<double, double>(h, h->L, h->L.val64, h->L.dinv64, r_dev, h->t64);
        solve<double, double>(h, h->U, h->U.val64, h->U.dinv64, h->t64, z_dev);
    }
    if (cudaGetLastError() != cudaSuccess) return LINA_GPU_ECUDA;
    const int e = read_err(h);
    if (e != 0) {
        lina::dev::set_error("ILU apply: a wait of the triangular solve ran out");
        if (e > 0) cudaMemset(h->err, 0, sizeof(int));
        return LINA_GPU_ECUDA;
    }
    return 0;
}
// reps applications (forward then backward triangular solve, no conversions) on a right-hand side of
// ones, CUDA events on the handle's stream around them: milliseconds per application
int lina_gpu_ilu_time_apply(lina_gpu_ilu* h, int precision, int reps, double* ms_per_apply) {
    if (!h || reps <= 0 || !ms_per_apply) return LINA_GPU_EINVAL;
    const int n = h->n;
    const int g = (int)std::min<long>(2048, (n + kT - 1) / kT);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return LINA_GPU_ECUDA;
    }
    if (precision == LINA_PREC_MIXED)
        fill_kernel<float><<<g, kT, 0, st()>>>(n, 1.0f, h->r32);
    else
        fill_kernel<double><<<g, kT, 0, st()>>>(n, 1.0, h->t64);
    double* r64 = h->t64;
    double* z64 = nullptr;
    if (precision != LINA_PREC_MIXED && cudaMalloc(&z64, 2 * (size_t)n * sizeof(double)) != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return LINA_GPU_ECUDA;
    }
    cudaEventRecord(e0, st());
    for (int k = 0; k < reps; k++) {
        if (precision == LINA_PREC_MIXED) {
            solve<float, float>(h, h->L, h->L.val32, h->L.dinv32, h->r32, h->t32);
            solve<float, float>(h, h->U, h->U.val32, h->U.dinv32, h->t32, h->z32);
        } else {
            solve<double, double>(h, h->L, h->L.val64, h->L.dinv64, r64, z64);
            solve<double, double>(h, h->U, h->U.val64, h->U.dinv64, z64, z64 + n);
        }
    }
    cudaEventRecord(e1, st());
    float ms = 0.f;
    const bool ok = cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (z64) cudaFree(z64);
    if (!ok || cudaGetLastError() != cudaSuccess) return LINA_GPU_ECUDA;
    const int e = read_err(h);
    if (e != 0) {
        lina::dev::set_error("ILU timing: a wait of the triangular solve ran out");
        if (e > 0) cudaMemset(h->err, 0, sizeof(int));
        return LINA_GPU_ECUDA;
    }
    *ms_per_apply = ms / reps;
    return 0;
}

}  // extern "C"
