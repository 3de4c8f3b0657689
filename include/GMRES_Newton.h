/*
 * GMRES_Newton.h - Newton solver with a finite-difference Jacobian and GMRES, and the
 * one-dimensional root finders, of the GB300 LinA library.
 * Same names and signatures as the reference header LinA/GMRES_Newton.h:21-36.
 */
#ifndef GMRES_NEWTON
#define GMRES_NEWTON

#include "itlin.h"
#include "linear_algebra.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LARGE_SYSTEM 1
#define SMALL_SYSTEM 0

/* Newton iteration for F(X) = B (Newton_set_function / Newton_set_inhomo) with the Jacobian
   J_ik = (F_i(X + h e_k) - F_i(X)) / h, h = 1e-6, on the nonzero pattern of Pattern; the step
   solves J d = B - F(X) by ILU(0)-preconditioned GMRES (LARGE_SYSTEM) or a sparse LU
   (SMALL_SYSTEM).  r0 < 0: the initial residual is computed.  Returns the Newton steps, or -1. */
int Newton_solver(sparse_matrix* Pattern, double* X, double maxiter, double eps, int mode, double r0);
/* repeated Newton_solver from the best of Newton_first_guess's random guesses, each root found
   deflating F for the next search; returns the number of roots (Newton_get_all_roots) */
int Newton_solver_mult_Root(sparse_matrix* Pattern, double maxiter, double eps, int mode);

void Newton_set_function(double (*F)(double* X, int i, int size));
void Newton_set_inhomo(double* B, int n);
void Newton_GMRES_options(int bases_imax, int maxiter, double tol);
void Newton_first_guess_options(int guess_num, int size, double* Min, double* Max);
void Newton_set_range(int size, double* Min, double* Max);
sparse_matrix* Newton_get_full_pattern(int size);
double** Newton_get_all_roots(void);
void Newton_first_guess(double* Res, int n);
int Newton_1D(double (*F)(double x), double** Roots, double min, double max, int max_iter, double eps);
int Interval_Separation_Newton_1D(double (*F)(double x), double** Roots, double min, double max, int max_iter,
                                  double eps, int int_num);
void set_RN_Hesse(sparse_matrix* A);
void set_RN_linear(double* B);

#ifdef __cplusplus
}
#endif

#endif
