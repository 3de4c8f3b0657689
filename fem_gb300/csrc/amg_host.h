// amg_host.h - host-side AMG hierarchy construction (setup phase) for the GB300 LinA library.
//
// The setup is a serial algorithm by definition in the reference (greedy C/F
// splitting driven by a max-priority queue), so it runs on the host here and
// produces CSR arrays that are uploaded once; the solve phase runs on the GPU.
// Every step reproduces the reference's integer output (labels, sparsity
// patterns) and its floating-point operation order, so that patterns and
// values agree bit for bit with LinA/Multigrid.c.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace lina {

// labels of LinA/Multigrid.h:23-27
enum { kUndecided = 0, kCoarse = 1, kFine = 2, kIsolated = 3 };
// coarsenings: the reference's (LinA/Multigrid.h:29-31) and PMIS on the GPU (this library's, opt-in)
enum { kAggressive = 1, kStandard = 2, kPmis = 3 };

struct Csr {
    int n = 0;      // rows
    int ncols = 0;  // columns (informational)
    std::vector<int> ptr{0};
    std::vector<int> col;
    std::vector<double> val;
    int64_t nnz() const { return (int64_t)col.size(); }
};

struct AmgParams {
    int dof = 1;
    int depth = 2;
    int smoothing_iterations = 2;
    int aggr_smoothing_iterations = 2;
    int coarsening = kStandard;   // kAggressive: finest level coarsened aggressively; kPmis: PMIS
                                  // labels on every level (gpu_pmis.cu)
    double eps_minus = 0.3;       // strength thresholds (Multigrid.c:35-36)
    double eps_plus = 0.5;
    double matrix_tol = 0.1;      // interpolation truncation (Multigrid.c:37)
    bool gpu_products = false;    // Galerkin products on the GPU (same results; host if it fails)
    int coarse_device_rows = 0;   // coarsest dense blocks of at least this many rows are left for the GPU
                                  // to invert (gpu_coarse.cu); 0: always inverted on the host
};

struct HostLevel {
    Csr A;                      // the level operator
    std::vector<int> labels;    // C/F/ISOLATED labels (levels >= 1)
    std::vector<int> dof_level; // which unknown (0..dof-1) each row belongs to
    Csr P;                      // prolongation (n x coarse_size), levels >= 1
    Csr R;                      // restriction (coarse_size x n), levels >= 1
    int coarse_size = 0;
};

struct CoarseSolver {
    int n = 0;                      // coarsest level size
    std::vector<int> block_rows;    // rows with more than one nonzero (dense block)
    std::vector<double> inv;        // dense inverse of the block, row-major, m x m (the block itself when
                                    // inverted is false: the GPU inverts it at upload)
    bool inverted = true;
    std::vector<double> diag_inv;   // 1/a_ii for rows outside the block (0 inside)
    std::vector<int> in_block;      // 1 if row is part of the dense block
    // a block-diagonal coarsest level (several independent systems): block k holds the block positions
    // [blocks[k], blocks[k+1]) with its inverse at inv[inv_offsets[k]], row-major; empty: one block
    std::vector<int> blocks;
    std::vector<long> inv_offsets;
    std::vector<char> block_inverted;  // per block (blocks non-empty): false = inverted at upload
};

struct HostHierarchy {
    AmgParams params;
    std::vector<HostLevel> lv;      // lv[depth-1] is the finest level
    std::vector<double> signs;      // make_positive_diag signs of the finest rows
    CoarseSolver coarse;
    std::string error;
};

// Build the full hierarchy (AMG_setup, LinA/Multigrid.c:1613-1754).  A is the
// caller's matrix in CSR with sorted columns (explicit zeros allowed).
// Returns false and sets h.error on a condition where the reference aborts.
bool amg_setup_host(const Csr& A, const AmgParams& p, HostHierarchy& h);

// Numeric re-setup with the P/R of an existing hierarchy
// (AMG_recompute_coarse_matrices, LinA/Multigrid.c:1756-1780).
bool amg_recompute_host(HostHierarchy& h, const Csr& A);

// Reference-semantics SpGEMM (sparse_product, LinA/linear_algebra.c:186-222).
Csr spgemm_ref(const Csr& A, const Csr& B);

// The same product on the GPU, bit-identical (gpu_spgemm.cu); false with err set if the device
// fails or a row has more distinct columns than its per-warp table.
bool spgemm_gpu(const Csr& A, const Csr& B, Csr& C, std::string& err);

// Hierarchy files: every level's A, P, R in the reference's write_sparse format
// (LinA/linear_algebra.c:832), labels and unknown numbers as int arrays, the
// parameters in a text header.  Loading recomputes the coarsest factorisation.
bool write_csr_file(const std::string& path, const Csr& A);
bool read_csr_file(const std::string& path, Csr& A, int ncols);
bool amg_save_host(const HostHierarchy& h, const std::string& dir, std::string& err);
// coarse_device_rows: as AmgParams::coarse_device_rows for the reloaded coarsest block
bool amg_load_host(const std::string& dir, HostHierarchy& h, int coarse_device_rows = 0);

// PMIS labels on the GPU (gpu_pmis.cu) from the strong-connection sets S (sptr, sidx) and their
// transpose T: label holds kIsolated / kCoarse for the points decided beforehand and kUndecided
// for the rest, and returns with every point decided.  False with err set if the device fails.
bool pmis_gpu(int n, const std::vector<int>& sptr, const std::vector<int>& sidx, const std::vector<int>& tptr,
              const std::vector<int>& tidx, std::vector<int>& label, std::string& err);

// Greedy first-fit colouring of the symmetric nonzero graph (smoother ordering).
int greedy_colouring(const Csr& A, std::vector<int>& colour);

}  // namespace lina
