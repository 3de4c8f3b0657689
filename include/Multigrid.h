/*
 * Multigrid.h - algebraic multigrid of the GB300 LinA library.
 *
 * Names, constants, types and signatures follow the reference header
 * LinA/Multigrid.h so that callers compile unchanged.  AMG_setup builds the
 * hierarchy on the host exactly as the reference does (same C/F splitting,
 * interpolation and Galerkin products) and uploads it to the GPU; AMG_solve
 * and every preconditioner application run their V-cycles on the GPU.
 */
#ifndef MULTI_H
#define MULTI_H

#include "PCGS.h"
#include "linear_algebra.h"

#ifdef __cplusplus
extern "C" {
#endif

#define NO 0
#define YES 1
#define UP 1
#define DOWN -1
#define NONE 0
#define LEFT 1
#define RIGHT 2
#define UNDECIDED 0
#define COARSE 1
#define FINE 2
#define ISOLATED 3
#define WEAK 4
#define DIRECT 1
#define STANDARD 2
#define AGGRESSIVE 1
#define WITHOUT_IOSOLATED 0
#define WITH_ISOLATED 1
#define STAND_ALONE 0
#define PREMODE 1
#define AMG_PCG 1
#define FULL_AMG 2
#define VARIABLE_SYSTEM_MATRIX 1
#define CONSTANT_SYSTEM_MATRIX 0

/* LinA/Multigrid.h:45-70 */
typedef struct AMG_SYSTEM_INFO {
    sparse_matrix** Coarse_A;
    sparse_matrix** Prolongation;
    sparse_matrix** Restriction;
    sparse_matrix** L;
    sparse_matrix** U;
    sparse_matrix* Signs;
    int** Coarsening;
    int* Fine_sizes;
    int* Coarse_sizes;
    int depth;
    int AMG_cycle_structure;
    int AMG_prolongation_method;
    int AMG_smoothing_iterations;
    int AMG_aggr_smoothing_iterations;
    int AMG_coarsening;
    int AMG_info;
    int AMG_deg_of_freedom;
    int (*F_Prolong)(sparse_matrix* A, sparse_matrix* B, int* Label, int i, int** Indices, double** Values,
                     int** Status, int** Strong, int** Positions);
    void (*AMG_coarsest_solver)(sparse_matrix* L, sparse_matrix* U, double* F, double* Sol, int size);
    int* (*Get_iter)(int depth);
} amg_system_info;

/* LinA/Multigrid.h:72-79 */
typedef struct AMG_STATISTICS {
    int calls;
    int max_iter;
    double max_res;
    int* Iterations;
    double* Residuals;
    char File_name[512];
} amg_statistics;

int AMG_solve(amg_system_info* Data, double* F, double* Fine_Sol, amg_statistics* Stat);
void AMG_recompute_coarse_matrices(amg_system_info* Info, sparse_matrix* New_matrix);
void AMG_SOR_smoother(sparse_matrix* A, double* F, double* Sol, int* Label, double alpha, int fix, int iter,
                      int deg_freedom);
void AMG_parallel_Jacobi_smoother(sparse_matrix* A, double* F, double* Sol, int* Label, double alpha, int fix,
                                  int iter, int deg_freedom);

amg_system_info* AMG_setup(sparse_matrix* A, int AMG_deg_of_freedom, int depth, int AMG_smoothing_iterations,
                           int AMG_aggr_smoothing_iterations, int AMG_coarsening, int AMG_cycle_structure,
                           int AMG_prolongation_method,
                           void (*AMG_coarsest_solver)(sparse_matrix* L, sparse_matrix* U, double* F, double* Sol,
                                                       int size),
                           int* (*Get_iter)(int depth));
int* AMG_default_iterations(int depth);
void AMG_print_info(int s);
void AMG_free_data(amg_system_info* Data);

/* Extensions without a counterpart in the reference.  PCG_set_AMG_data selects the hierarchy (from
   AMG_setup) that PCG_AMG_vcycle_precon applies: one V-cycle from the zero guess, Z = M^-1 R (AMG_solve
   with one cycle and a zeroed Z).  When a caller installs PCG_default(A, ...) (the operator PCG_mult)
   and PCG_set_precon(PCG_AMG_vcycle_precon) for a hierarchy built by AMG_setup from the same A (the same
   pointer, unchanged since AMG_setup or AMG_recompute_coarse_matrices), pcg runs its whole loop on the
   GPU as one captured graph: the reference's stopping rule ||R|| / ||M^-1 R_0||, X as initial guess,
   get_pcg_residuum as the reference defines it; in mixed precision (AMG_gpu_set_precision(1)) the
   iteration is the truncated flexible CG of lina_gpu_pcg. */
void PCG_set_AMG_data(amg_system_info* data);
int PCG_AMG_vcycle_precon(int n, double* R, double* Z);
void AMG_set_SOR_relaxation_coeff(double alpha);
void set_connection_thresholds(double negative, double positive);

void AMG_set_eps(double eps);
void AMG_set_max_iter(int iter);
void AMG_set_deg_of_freedom(int n);
void AMG_set_matrix_tolerance(double tol);
void AMG_set_smoother(void (*Smoother)(sparse_matrix* A, double* F, double* Sol, int* Label, double alpha, int fix,
                                       int iter, int deg_freedom));
int AMG_info_set(void);
int AMG_get_max_iter(void);

amg_statistics AMG_init_stat(const char* Out);
void AMG_add_stat(amg_statistics* Stat, int iter, double res);
void AMG_print_stat(amg_statistics* Stat);

/* ---- additions of the GB300 library (no counterpart in the reference) ---- */
/* damped Jacobi smoother x <- x + alpha D^-1 (F - A x); install with AMG_set_smoother */
void AMG_damped_Jacobi_smoother(sparse_matrix* A, double* F, double* Sol, int* Label, double alpha, int fix,
                                int iter, int deg_freedom);
/* precision of the GPU V-cycle: 0 FP64 (default), 1 FP32 (mixed precision) */
void AMG_gpu_set_precision(int precision);

#ifdef __cplusplus
}
#endif

#endif
