// gpu_pmis.cu - PMIS coarsening on the GPU: an opt-in alternative (coarsening LINA_PMIS) to the
// reference's sequential greedy AMG_coarsener (LinA/Multigrid.c:377-473).  Its labels differ from
// the reference's; everything after the labels (coarse numbering, interpolation, Galerkin
// products) is the reference's algorithm as for the other coarsenings.
//
// The method is the parallel modified independent set of De Sterck, Yang and Heys ("Reducing
// complexity in parallel algebraic multigrid preconditioners", SIAM J. Matrix Anal. Appl. 27,
// 2006), on the strong-connection sets S_i (the points i depends on strongly, same unknown only)
// and their transpose T_i (the points that depend on i strongly):
//  * measure m_i = |T_i| + r_i, with r_i in [0, 1) from an integer hash of i (the same every run);
//    ties between equal measures go to the larger index;
//  * points nothing depends on strongly (|T_i| = 0) become fine at once;
//  * then, until no point is undecided: every undecided point whose measure exceeds that of all
//    its undecided neighbours in S_i and T_i becomes coarse, and every undecided point that depends
//    strongly on a coarse point becomes fine;
//  * last, a fine point without a coarse point in S_i becomes coarse, so that every fine row of
//    the interpolation has a strong coarse neighbour.
// Coarse points selected in the loop are independent in the symmetrised strength graph.  Each pass
// reads the labels of the previous one only (the new labels go to a second array), so the result
// does not depend on the order in which threads run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "amg_host.h"
#include "gpu_ops.h"

namespace lina {
namespace {

constexpr int kT = 256;

cudaStream_t st() { return (cudaStream_t)lina::dev::stream(); }

int grid(long n) { return (int)std::max(1L, std::min(4096L, (n + kT - 1) / kT)); }

// the 32-bit finaliser of MurmurHash3 (a public-domain integer mix)
__host__ __device__ inline unsigned mix32(unsigned h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ double measure(int i, const int* __restrict__ tptr) {
    return (double)(tptr[i + 1] - tptr[i]) + (double)(mix32((unsigned)i) >> 8) * (1.0 / 16777216.0);
}

// (m_a, a) > (m_b, b)
__device__ __forceinline__ bool above(double ma, int a, double mb, int b) { return ma > mb || (ma == mb && a > b); }

__global__ void init_kernel(int n, const int* __restrict__ tptr, const int* __restrict__ label_in, int* label) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int l = label_in[i];
        if (l == kUndecided && tptr[i + 1] == tptr[i]) l = kFine;
        label[i] = l;
    }
}

// undecided points that are local maxima of the measure among their undecided strong neighbours
__global__ void select_kernel(int n, const int* __restrict__ sptr, const int* __restrict__ sidx,
                              const int* __restrict__ tptr, const int* __restrict__ tidx,
                              const int* __restrict__ label, int* __restrict__ next) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int l = label[i];
        if (l == kUndecided) {
            const double mi = measure(i, tptr);
            bool top = true;
            for (int p = sptr[i]; p < sptr[i + 1] && top; p++) {
                const int j = sidx[p];
                if (label[j] == kUndecided && !above(mi, i, measure(j, tptr), j)) top = false;
            }
            for (int p = tptr[i]; p < tptr[i + 1] && top; p++) {
                const int j = tidx[p];
                if (label[j] == kUndecided && !above(mi, i, measure(j, tptr), j)) top = false;
            }
            if (top) l = kCoarse;
        }
        next[i] = l;
    }
}

// undecided points that depend strongly on a coarse point become fine; counts the rest
__global__ void fine_kernel(int n, const int* __restrict__ sptr, const int* __restrict__ sidx,
                            const int* __restrict__ label, int* __restrict__ next, unsigned* undecided) {
    unsigned left = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int l = label[i];
        if (l == kUndecided) {
            for (int p = sptr[i]; p < sptr[i + 1]; p++)
                if (label[sidx[p]] == kCoarse) {
                    l = kFine;
                    break;
                }
            if (l == kUndecided) left++;
        }
        next[i] = l;
    }
    if (left) atomicAdd(undecided, left);
}

// fine points without a coarse point among the points they depend on strongly become coarse
__global__ void fixup_kernel(int n, const int* __restrict__ sptr, const int* __restrict__ sidx,
                             const int* __restrict__ label, int* __restrict__ next) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int l = label[i];
        if (l == kFine && sptr[i + 1] > sptr[i]) {
            bool has = false;
            for (int p = sptr[i]; p < sptr[i + 1] && !has; p++) has = label[sidx[p]] == kCoarse;
            if (!has) l = kCoarse;
        }
        next[i] = l;
    }
}

}  // namespace

bool pmis_gpu(int n, const std::vector<int>& sptr, const std::vector<int>& sidx, const std::vector<int>& tptr,
              const std::vector<int>& tidx, std::vector<int>& label, std::string& err) {
    if (n <= 0) return true;
    if (!lina::dev::ready()) {
        err = "PMIS coarsening: no CUDA device";
        return false;
    }
    int *dsp = nullptr, *dsi = nullptr, *dtp = nullptr, *dti = nullptr, *la = nullptr, *lb = nullptr;
    unsigned* cnt = nullptr;
    auto up = [&](int** d, const std::vector<int>& h) {
        if (cudaMalloc(d, std::max<size_t>(h.size(), 1) * sizeof(int)) != cudaSuccess) return false;
        return h.empty() || cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, st()) ==
                                cudaSuccess;
    };
    bool ok = up(&dsp, sptr) && up(&dsi, sidx) && up(&dtp, tptr) && up(&dti, tidx) && up(&la, label) &&
              cudaMalloc(&lb, (size_t)n * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&cnt, sizeof(unsigned)) == cudaSuccess;
    if (ok) {
        init_kernel<<<grid(n), kT, 0, st()>>>(n, dtp, la, lb);
        std::swap(la, lb);
        // every round decides at least the undecided point of largest measure
        unsigned left = 1;
        for (int round = 0; ok && left > 0; round++) {
            if (round > n) {
                err = "PMIS coarsening did not finish";
                ok = false;
                break;
            }
            select_kernel<<<grid(n), kT, 0, st()>>>(n, dsp, dsi, dtp, dti, la, lb);
            std::swap(la, lb);
            ok = cudaMemsetAsync(cnt, 0, sizeof(unsigned), st()) == cudaSuccess;
            fine_kernel<<<grid(n), kT, 0, st()>>>(n, dsp, dsi, la, lb, cnt);
            std::swap(la, lb);
            ok = ok && cudaMemcpyAsync(&left, cnt, sizeof(unsigned), cudaMemcpyDeviceToHost, st()) == cudaSuccess &&
                 cudaStreamSynchronize(st()) == cudaSuccess;
        }
        if (ok) {
            fixup_kernel<<<grid(n), kT, 0, st()>>>(n, dsp, dsi, la, lb);
            std::swap(la, lb);
            ok = cudaMemcpyAsync(label.data(), la, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st()) ==
                     cudaSuccess &&
                 cudaStreamSynchronize(st()) == cudaSuccess && cudaGetLastError() == cudaSuccess;
        }
        if (!ok && err.empty()) err = "PMIS coarsening: CUDA error";
    } else {
        err = "PMIS coarsening: device allocation failed";
    }
    for (void* p : {(void*)dsp, (void*)dsi, (void*)dtp, (void*)dti, (void*)la, (void*)lb, (void*)cnt})
        if (p) cudaFree(p);
    return ok;
}

}  // namespace lina
