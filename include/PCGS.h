/*
 * PCGS.h - preconditioned conjugate gradients of the GB300 LinA library.
 *
 * Same names and signatures as the reference header LinA/PCGS.h.  pcg runs
 * its vector operations on the GPU; when the installed operators are the
 * library's own (PCG_default with PCG_mult, PCG_set_AMG_preconditioner, the
 * ILU preconditioner of PCG_set_default_precon) they run on the GPU too, and a
 * caller's own callbacks are called on host copies of the vectors.
 */
#ifndef PCGS_H
#define PCGS_H

#include "linear_algebra.h"
#include "Multigrid.h"

#ifdef __cplusplus
extern "C" {
#endif

int pcg(double* X, double* B, int n, double tol, int max_iter);
double get_pcg_residuum(void);

void PCG_set_precon(int (*Precon)(int n, double* R, double* Z));
void PCG_set_mat_mult(void (*Mat_mult)(int n, double* x, double* y));
void* PCG_get_precon(void);
void* PCG_get_mat_mult(void);
void PCG_set_default_precon(void);
void PCG_default(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U);
void PCG_set_AMG_preconditioner(sparse_matrix* A, int num_fields, int depth);

/* the library's own operators (installed by the functions above) */
void PCG_mult(int n, double* y, double* z);
int PCG_preconlr(int n, double* z, double* w);
int PCG_AMG_precon(int n, double* Y, double* X);

/* PCG_set_AMG_data and PCG_AMG_vcycle_precon (extensions for pcg on the device) are declared in
   Multigrid.h, after the hierarchy type. */

#ifdef __cplusplus
}
#endif

#endif
