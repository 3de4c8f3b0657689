// gpu_spgemm.cu - sparse matrix product on the GPU with the reference's
// sparse_product semantics (LinA/linear_algebra.c:186-222), for the Galerkin
// products R (A P) of the AMG hierarchy.
//
// The reference builds row i of C = A B by walking A's row i in stored order
// and, for every nonzero a_ik, B's row k in stored order: a product with a
// nonzero b_kj starts column j or is added to it (row i starts with the entry
// (i, 0.0)), the row is sorted by column, and delete_zeros drops exact zeros
// (a row left empty keeps (i, 0.0)).  Each output entry is therefore a sum in
// a fixed order.  Here one warp builds one output row in a hash table in
// shared memory: the warp walks A's row like the reference, and the lanes
// take B's row k together; the columns of one row of B are distinct, so no
// two lanes touch the same entry in one step, and the warp synchronises
// between rows of B, so every entry receives its terms in the reference's
// order (products and sums rounded one by one: bit-identical to the host
// restatement spgemm_ref).  Two passes: row lengths, then the rows.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <string>
#include <vector>

#include "amg_host.h"
#include "gpu_ops.h"
#include "lina_gpu.h"

namespace lina {
namespace {

constexpr int kWarps = 4;                    // warps per block, one output row each
constexpr int kTable = 1024;                 // hash slots per warp (power of two)
constexpr int kFill = kTable / 2;            // more distinct columns in one row: overflow
constexpr int kSmem = kWarps * kTable * 24;  // keys, values, compacted keys and values

cudaStream_t st() { return (cudaStream_t)lina::dev::stream(); }

__device__ __forceinline__ int slot_of(int j) { return (int)(((unsigned)j * 2654435761u) >> 22) & (kTable - 1); }

// pass 0 (WRITE false): row lengths after delete_zeros into len[i]; pass 1: the rows at Cp[i]
template <bool WRITE>
__global__ void __launch_bounds__(kWarps * 32) spgemm_kernel(int n, const int* __restrict__ Ap,
                                                             const int* __restrict__ Ac, const double* __restrict__ Av,
                                                             const int* __restrict__ Bp, const int* __restrict__ Bc,
                                                             const double* __restrict__ Bv, int* __restrict__ len,
                                                             const int* __restrict__ Cp, int* __restrict__ Cc,
                                                             double* __restrict__ Cv, int* overflow) {
    extern __shared__ unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int* key = (int*)smem + w * kTable;
    double* val = (double*)(smem + (size_t)kWarps * kTable * 4) + w * kTable;
    int* ckey = (int*)(smem + (size_t)kWarps * kTable * 12) + w * kTable;
    double* cval = (double*)(smem + (size_t)kWarps * kTable * 16) + w * kTable;
    __shared__ int claimed[kWarps];
    const long gw = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long row = gw; row < n; row += nw) {
        const int i = (int)row;
        for (int s = lane; s < kTable; s += 32) key[s] = -1;
        if (lane == 0) claimed[w] = 0;
        __syncwarp();
        if (lane == 0) {  // the row starts as (i, 0.0)
            int s = slot_of(i);
            while (key[s] != -1) s = (s + 1) & (kTable - 1);
            key[s] = i;
            val[s] = 0.0;
            claimed[w] = 1;
        }
        __syncwarp();
        bool bad = false;
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const double a = Av[p];
            if (a == 0.0) continue;
            const int k = Ac[p];
            for (int r = Bp[k] + lane; r < Bp[k + 1]; r += 32) {
                const double b = Bv[r];
                if (b == 0.0) continue;
                const int j = Bc[r];
                const double prod = __dmul_rn(a, b);
                int s = slot_of(j);
                for (int probe = 0;; probe++) {
                    const int old = atomicCAS(&key[s], -1, j);
                    if (old == -1) {
                        val[s] = prod;
                        if (atomicAdd(&claimed[w], 1) >= kFill) bad = true;
                        break;
                    }
                    if (old == j) {
                        val[s] = __dadd_rn(val[s], prod);
                        break;
                    }
                    s = (s + 1) & (kTable - 1);
                    if (probe >= kTable) {
                        bad = true;
                        break;
                    }
                }
            }
            __syncwarp();
        }
        if (__any_sync(0xffffffffu, bad)) {
            if (lane == 0) {
                atomicExch(overflow, 1);
                if (!WRITE) len[i] = 1;
            }
            __syncwarp();
            continue;
        }
        // compact the table
        int m = 0;
        for (int s0 = 0; s0 < kTable; s0 += 32) {
            const int s = s0 + lane;
            const bool occ = key[s] >= 0;
            const unsigned bal = __ballot_sync(0xffffffffu, occ);
            if (occ) {
                const int pos = m + __popc(bal & ((1u << lane) - 1u));
                ckey[pos] = key[s];
                cval[pos] = val[s];
            }
            m += __popc(bal);
        }
        __syncwarp();
        // delete_zeros: rows of more than one entry lose their zeros; an emptied row is (i, 0.0)
        int kept = m;
        if (m > 1) {
            kept = 0;
            for (int e = lane; e < m; e += 32) kept += (cval[e] != 0.0) ? 1 : 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
        }
        if (!WRITE) {
            if (lane == 0) len[i] = kept > 0 ? kept : 1;
        } else if (kept == 0) {
            if (lane == 0) {
                Cc[Cp[i]] = i;
                Cv[Cp[i]] = 0.0;
            }
        } else {
            const bool filter = m > 1;
            for (int e = lane; e < m; e += 32) {
                const double v = cval[e];
                if (filter && v == 0.0) continue;
                const int c = ckey[e];
                int rank = 0;
                for (int f = 0; f < m; f++)
                    if (ckey[f] < c && !(filter && cval[f] == 0.0)) rank++;
                Cc[Cp[i] + rank] = c;
                Cv[Cp[i] + rank] = v;
            }
        }
        __syncwarp();
    }
}

struct DevBuf {
    std::vector<void*> p;
    template <typename T>
    T* get(size_t count) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        p.push_back(q);
        return (T*)q;
    }
    ~DevBuf() {
        cudaStreamSynchronize(st());
        for (void* q : p) cudaFree(q);
    }
};

template <typename T>
bool put(T* d, const std::vector<T>& h) {
    return h.empty() || cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st()) == cudaSuccess;
}

}  // namespace

// C = A B on the GPU (sparse_product semantics); false with err set on a device failure or a row
// with more distinct columns than the per-warp table holds (the caller then uses spgemm_ref)
bool spgemm_gpu(const Csr& A, const Csr& B, Csr& C, std::string& err) {
    if (!lina::dev::ready()) {
        err = "no GPU";
        return false;
    }
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(spgemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem) !=
                cudaSuccess ||
            cudaFuncSetAttribute(spgemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem) !=
                cudaSuccess) {
            err = "spgemm: shared memory attribute refused";
            return false;
        }
        attr = true;
    }
    const int n = A.n;
    DevBuf buf;
    int *Ap = buf.get<int>(A.ptr.size()), *Ac = buf.get<int>(A.col.size()), *Bp = buf.get<int>(B.ptr.size()),
        *Bc = buf.get<int>(B.col.size()), *len = buf.get<int>(n), *ovf = buf.get<int>(1);
    double *Av = buf.get<double>(A.val.size()), *Bv = buf.get<double>(B.val.size());
    if (!Ap || !Ac || !Bp || !Bc || !len || !ovf || !Av || !Bv || !put(Ap, A.ptr) || !put(Ac, A.col) ||
        !put(Av, A.val) || !put(Bp, B.ptr) || !put(Bc, B.col) || !put(Bv, B.val) ||
        cudaMemsetAsync(ovf, 0, sizeof(int), st()) != cudaSuccess) {
        err = "spgemm: device allocation or upload failed";
        return false;
    }
    const int threads = kWarps * 32;
    const long blocks = std::min<long>(((long)n + kWarps - 1) / kWarps, 152L * 16);
    spgemm_kernel<false><<<(int)std::max(1L, blocks), threads, kSmem, st()>>>(n, Ap, Ac, Av, Bp, Bc, Bv, len, nullptr,
                                                                             nullptr, nullptr, ovf);
    std::vector<int> hl(n);
    int hovf = 0;
    if (cudaGetLastError() != cudaSuccess ||
        (n && cudaMemcpyAsync(hl.data(), len, n * sizeof(int), cudaMemcpyDeviceToHost, st()) != cudaSuccess) ||
        cudaMemcpyAsync(&hovf, ovf, sizeof(int), cudaMemcpyDeviceToHost, st()) != cudaSuccess ||
        cudaStreamSynchronize(st()) != cudaSuccess) {
        err = "spgemm: row-length pass failed";
        return false;
    }
    if (hovf) {
        err = "spgemm: a row has more distinct columns than the device table";
        return false;
    }
    C = Csr();
    C.n = n;
    C.ncols = B.ncols;
    C.ptr.assign(n + 1, 0);
    for (int i = 0; i < n; i++) {
        if ((long)C.ptr[i] + hl[i] > INT_MAX) {
            err = "spgemm: product too large for 32-bit offsets";
            return false;
        }
        C.ptr[i + 1] = C.ptr[i] + hl[i];
    }
    const long nnz = C.ptr[n];
    int *Cp = buf.get<int>(n + 1), *Cc = buf.get<int>(nnz);
    double* Cv = buf.get<double>(nnz);
    if (!Cp || !Cc || !Cv || !put(Cp, C.ptr)) {
        err = "spgemm: device allocation failed";
        return false;
    }
    spgemm_kernel<true><<<(int)std::max(1L, blocks), threads, kSmem, st()>>>(n, Ap, Ac, Av, Bp, Bc, Bv, nullptr, Cp, Cc,
                                                                            Cv, ovf);
    C.col.resize(nnz);
    C.val.resize(nnz);
    if (cudaGetLastError() != cudaSuccess ||
        (nnz && cudaMemcpyAsync(C.col.data(), Cc, nnz * sizeof(int), cudaMemcpyDeviceToHost, st()) != cudaSuccess) ||
        (nnz && cudaMemcpyAsync(C.val.data(), Cv, nnz * sizeof(double), cudaMemcpyDeviceToHost, st()) != cudaSuccess) ||
        cudaStreamSynchronize(st()) != cudaSuccess) {
        err = "spgemm: row pass failed";
        return false;
    }
    return true;
}

}  // namespace lina

// ---------------------------------------------------------------- C-ABI
extern "C" int lina_gpu_spgemm(int n, int ncols_b, const int* Ap, const int* Ac, const double* Av, int nb,
                               const int* Bp, const int* Bc, const double* Bv, long capacity, int* Cp, int* Cc,
                               double* Cv, long* nnz) {
    if (n < 0 || nb < 0 || !Ap || !Bp || !nnz || (capacity > 0 && (!Cp || !Cc || !Cv))) {
        lina::dev::set_error("lina_gpu_spgemm: invalid argument");
        return LINA_GPU_EINVAL;
    }
    lina::Csr A, B, C;
    A.n = n;
    A.ncols = nb;
    A.ptr.assign(Ap, Ap + n + 1);
    A.col.assign(Ac, Ac + Ap[n]);
    A.val.assign(Av, Av + Ap[n]);
    B.n = nb;
    B.ncols = ncols_b;
    B.ptr.assign(Bp, Bp + nb + 1);
    B.col.assign(Bc, Bc + Bp[nb]);
    B.val.assign(Bv, Bv + Bp[nb]);
    for (int c : A.col)
        if (c < 0 || c >= nb) {
            lina::dev::set_error("lina_gpu_spgemm: a column of A is not a row of B");
            return LINA_GPU_EINVAL;
        }
    std::string err;
    if (!lina::spgemm_gpu(A, B, C, err)) {
        lina::dev::set_error(("lina_gpu_spgemm: " + err).c_str());
        return LINA_GPU_ECUDA;
    }
    *nnz = C.nnz();
    if (capacity < C.nnz()) {
        if (capacity > 0) {
            lina::dev::set_error("lina_gpu_spgemm: output capacity too small");
            return LINA_GPU_EINVAL;
        }
        return 0;
    }
    std::copy(C.ptr.begin(), C.ptr.end(), Cp);
    std::copy(C.col.begin(), C.col.end(), Cc);
    std::copy(C.val.begin(), C.val.end(), Cv);
    return 0;
}
