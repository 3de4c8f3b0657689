/*
 * GMRES_Newton.h - Newton and one-dimensional root finders of the GB300 LinA library.
 * Same names and signatures as the reference header LinA/GMRES_Newton.h; the
 * one-dimensional finders (GMRES_Newton.c:353-440) are what reflective Newton uses.
 */
#ifndef GMRES_NEWTON
#define GMRES_NEWTON

#include "linear_algebra.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LARGE_SYSTEM 1
#define SMALL_SYSTEM 0

int Newton_1D(double (*F)(double x), double** Roots, double min, double max, int max_iter, double eps);
int Interval_Separation_Newton_1D(double (*F)(double x), double** Roots, double min, double max, int max_iter,
                                  double eps, int int_num);
void set_RN_Hesse(sparse_matrix* A);
void set_RN_linear(double* B);

#ifdef __cplusplus
}
#endif

#endif
