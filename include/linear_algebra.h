/*
 * linear_algebra.h - the LinA row-list sparse matrix type and the helpers the
 * solve path and its callers use (GB300 LinA library).
 *
 * Declarations keep the names, argument order and meaning of the reference
 * header LinA/linear_algebra.h so that callers compile and link unchanged.
 * The matrix type is the reference's (LinA/linear_algebra.h:29-34): row i
 * holds Len[i] entries, columns sorted increasingly in Indices[i], values in
 * Values[i]; a row without entries holds the single entry (i, 0.0).
 *
 * Only the part of the reference header that belongs to the sparse solve path
 * and to the matrix helpers its callers (Crack/crack.c, FEM2D/FEM.c) use is
 * provided; the 3-tensor, general-rank, Arnoldi/QR/Ritz, UMFPACK-conversion
 * and file I/O utilities of the reference header are not part of this library.
 */
#ifndef LINEAR_ALGEBRA_H
#define LINEAR_ALGEBRA_H

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AUTOMATIC -1
#define INIT NULL
#define NEG_DEFINITE -1.
#define POS_DEFINITE 1.
#define ASS_FLUX 1
#define ASS_DEFAULT 0

/* LinA/linear_algebra.h:29-34 */
typedef struct SPARSE {
    double** Values;
    int** Indices;
    int* Len;
    int size;
} sparse_matrix;

/* LinA/linear_algebra.h:90-97 (state of active_set_solver) */
typedef struct ASS_IFO {
    int active_size;
    int* Active;
    double* Signs;
    double* Constraint;
    int* Iter_history;
    int calls;
} ass_info;

/* ---- matrix construction and access (linear_algebra.c:484-1300) ---- */
sparse_matrix* sparse_zero(int length);
sparse_matrix* sparse_identity(int length);
sparse_matrix* sparse_diagonal(double* d, int n);
sparse_matrix* clone(sparse_matrix* A);
void Free_sparse(sparse_matrix* A);
int insert_sparse(sparse_matrix* A, double a, int i, int j);
void set_sparse(sparse_matrix* A, double a, int i, int j);
void insert_element_at(sparse_matrix* A, double a, int i, int j, int pos);
void remove_element_at(sparse_matrix* A, int i, int pos);
void remove_element(sparse_matrix* A, int i, int j);
void reset_row(sparse_matrix* A, int i);
void delete_zeros(sparse_matrix* A);
void remove_zero(sparse_matrix* A, int i);
void remove_zeros(sparse_matrix* A);
int get_position(int* list, int size, int val, int* Flag);
double get_matrix_element(sparse_matrix* A, int i, int j);
double get_diag(sparse_matrix* A, int i);
sparse_matrix* get_transpose(sparse_matrix* A, int new_size);
/* binary matrix files (write_sparse / read_sparse, LinA/linear_algebra.c:832-869): the file
   path/name holds int n, int Len[n], every row's indices, every row's values; 1 / a new matrix on
   success, 0 / NULL otherwise */
int write_sparse(sparse_matrix* A, char* path, char* name);
sparse_matrix* read_sparse(char* path, char* name);
void sparse_add(sparse_matrix* A, sparse_matrix* B, double factor);
sparse_matrix* sparse_product(sparse_matrix* A, sparse_matrix* B);
double* sparse_row_sum(sparse_matrix* A);
void scalar_sparse_mult(double a, sparse_matrix* A);
sparse_matrix* make_positive_diag(sparse_matrix* A);
int diag_zero(sparse_matrix* A);
sparse_matrix* Lap_2D_Dirichlet(double a, double b, int dom_size);

/* ---- products (linear_algebra.c:134-186, :442) ---- */
double* sparse_mult(sparse_matrix* A, double* x);
void linear_map(double* x, double fac, sparse_matrix* A, double* y);
void sparse_multiplication(sparse_matrix* A, double* x);
double sparse_bilinear(double* y, sparse_matrix* A, double* x);

/* ---- vectors (linear_algebra.c:56-317, :3158) ---- */
int min(int a, int b);
int max(int a, int b);
double* zero_vector(int n);
double* clone_vector(double* x, int n);
void copy_vector_to(double* x, double* y, int n);
double scalar(double* x1, double* x2, int n);
double euklid_norm(double* x1, int n);
void scalar_mult(double a, double* x, int n);
void vector_add(double* x, double* y, double factor, int n);

int* zero_int_list(int n);
int* clone_list(int* x, int n);
double* generate_vector(int size, double val);
void copy_vector_content(double* x, double* y, int x_pos, int y_pos, int size);
void vector_pseudo_mult(double* x, double* y, int n);
void enlarge_matrix(sparse_matrix* A, int mesh_size, int new_size, int equ_index, int var_index);
void simple_enlarge_matrix(sparse_matrix* A, int add_size);

/* ---- complete factorisations (linear_algebra.c:2909, :3040, :3122) ---- */
void LU_factorzation(double** A, double** L, double** U, int size);
void sparse_LU_factorization(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U);
void complete_LU_factorization(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U);

/* ---- active-set solver (linear_algebra.c:4923-5042): KKT loop around the caller's Solver ---- */
int active_set_solver(sparse_matrix* A, double* Sol, double* b, sparse_matrix* B, double* L, double* U,
                      int (*Solver)(sparse_matrix* A, double* X, double* b), int max_iter, double definiteness,
                      int mode, ass_info** solver_info);
void free_ass_info(ass_info** info);

/* Local solvers on the GPU for the slots that take int f(sparse_matrix* A, double* X, double* b):
   reflective_newton's RN_set_local_solver, active_set_solver's Solver, and a replacement for
   Crack/crack.c's UMFPACK wrapper multifrontal_solver.  No counterpart in the reference.  Both return
   POSITIVE_DEFINITE (1) when the solve reached its tolerance, INDEFINITE (0) otherwise.
   LinA_gpu_spd_solver: symmetric positive definite A, AMG-preconditioned CG (hierarchy kept between calls,
   coarse levels recomputed when only the values change), X as initial guess, ||b - A X|| <= 1e-10 ||b||.
   LinA_gpu_general_solver: any square A (e.g. active-set KKT systems), GMRES(30) with ILU(0) of A (none on
   a zero pivot), from X = 0, relative residual 1e-10. */
int LinA_gpu_spd_solver(sparse_matrix* A, double* X, double* b);
int LinA_gpu_general_solver(sparse_matrix* A, double* X, double* b);

/* ---- incomplete factorisation and triangular solves (linear_algebra.c:1952-2043) ---- */
int incomplete_LU_factorization(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U);
void L_triang_invert(sparse_matrix* L, double* x);
void U_triang_invert(sparse_matrix* U, double* x);
double matrix_residuum(sparse_matrix* A, double* Sol, double* b);
double ILU_residuum(sparse_matrix* A, sparse_matrix* L, sparse_matrix* U, double* Sol, double* b);

#ifdef __cplusplus
}
#endif

#define free_sparse(A) \
    Free_sparse(A);    \
    free(A)

#endif
