/*
 * itlin.h - option and result records of the GMRES entry point of the GB300
 * LinA library.
 *
 * The reference links the ZIB NewtonLib GMRES (LinA/gmres.c, declared with
 * the records of LinA/itlin.h:58-84); callers such as FEM2D/FEM.c:739 fill an
 * ITLIN_OPT, call gmres() and read ITLIN_INFO.  The record layouts, enum values
 * and the gmres() signature below are that calling contract; the solver
 * behind them is this library's own (fem_gb300/csrc/gmres_newton.cpp).
 */
#ifndef ITLIN_H
#define ITLIN_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { None = 0, Minimum = 1, Verbose = 2, Debug = 3 } PRINT_LEVEL;
typedef enum { False = 0, True = 1 } LOGICAL;
typedef enum { CheckOnRestart = 0, CheckEachIter = 1 } TERM_CHECK;
typedef enum { Absolute = 0, Relative = 1 } CONV_CHECK;

typedef void MATVEC(int, double*, double*);
typedef void PRECON(int, double*, double*);

struct ITLIN_OPT {
    double tol, rho;
    int i_max, maxiter;
    TERM_CHECK termcheck; /* GMRES: test the residual at every step or at restarts only */
    CONV_CHECK convcheck; /* unused by GMRES */
    LOGICAL rescale;      /* unused by GMRES */
    PRINT_LEVEL errorlevel, monitorlevel, datalevel;
    FILE *errorfile, *monitorfile, *datafile, *iterfile, *resfile, *miscfile;
    double* scale;
};

struct ITLIN_INFO {
    double precision, normdx, residuum;
    int iter, rcode, subcode, nomatvec, noprecon, noprecl, noprecr;
};

/* Restarted GMRES on B_l A B_r y = b from the initial y: y is the right-preconditioned iterate
   (the caller forms x = B_r y).  Stops when ||b - B_l A B_r y|| / ||b - B_l A B_r y_0|| <= opt->tol
   (clamped to [1e-15, 0.1]) or after opt->maxiter steps (default 100), checked at every step
   (CheckEachIter) or at restarts; restarts every opt->i_max steps (default min(10, n)).
   info->rcode: 0 converged, 2 step limit, 1 singular Hessenberg system, 20 n <= 0,
   21 tol <= 0, -99 no matvec.  Products and preconditioners that are the library's own
   (PCG_mult, RN_default_mat_mult, PCG_preconlr, PCG_AMG_precon, BI_AMG_precon) run on the GPU;
   other callbacks run on host copies. */
void gmres(int n, double* y, MATVEC* matvec, PRECON* preconr, PRECON* preconl, double* b, struct ITLIN_OPT* opt,
           struct ITLIN_INFO* info);

#ifdef __cplusplus
}
#endif

#endif
