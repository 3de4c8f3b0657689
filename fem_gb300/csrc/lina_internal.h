// lina_internal.h - helpers shared by the drop-in API translation units (internal).
#pragma once

#include <cstdint>
#include <vector>

#include "lina_gpu.h"
#include "linear_algebra.h"

namespace lina {
namespace api {

// a row-list matrix laid out as CSR (columns and values in row order)
struct CsrCopy {
    int n = 0;
    std::vector<int> ptr, col;
    std::vector<double> val;
};

CsrCopy to_csr(const sparse_matrix* A);
// a new row-list matrix from CSR (an empty row becomes the reference's (i, 0.0))
sparse_matrix* from_csr(int n, const int* ptr, const int* col, const double* val);
// content fingerprint: decides whether a cached device copy is still current
uint64_t fingerprint(const sparse_matrix* A);
// device copy of a caller matrix, cached by pointer and fingerprint
lina_gpu_matrix* device_matrix(const sparse_matrix* A);
// drop the cached device copy of a matrix that is about to be freed
void forget_device_matrix(const sparse_matrix* A);
// device ILU(0) solves for factors in the reference's layout, cached likewise
lina_gpu_ilu* device_ilu(const sparse_matrix* L, const sparse_matrix* U);
// BiCGStab settings (BI_set_eps / BI_set_max_iter)
double bi_eps_value();
// the matrix RN_default_mat_mult multiplies with (RN_set_default_matrix)
sparse_matrix* rn_default_matrix();

// callbacks of the reference's solver interfaces applied to device vectors: the library's own
// products and preconditioners (PCG_mult, RN_default_mat_mult, PCG_preconlr, PCG_AMG_precon,
// BI_AMG_precon) run on the GPU, any other function on host copies
using MatMultFn = void (*)(int, double*, double*);
using PreconFn = int (*)(int, double*, double*);
bool device_matmult(MatMultFn f, int n, const double* x, double* y);
int device_precon(PreconFn f, int n, const double* r, double* z);

}  // namespace api
}  // namespace lina
