/*
 * lina_port.h - CPU restatement of the reference LinA solve phase (ORACLE).
 *
 * Test infrastructure: the GPU library never links this.  Tests use it as an
 * independent CPU checker; bench.py times it as the CPU baseline on hosts
 * where the reference itself cannot be built.  It restates, on CSR arrays:
 *   - the V-cycle AMG_V_cycle            (LinA/Multigrid.c:1536-1580)
 *   - one AMG_solve application          (LinA/Multigrid.c:1863-1931)
 *     with AMG_fix_isolated              (LinA/Multigrid.c:1301-1319)
 *   - the coarsest direct solve          (sparse_LU_factorization,
 *                                          LinA/linear_algebra.c:3040, LU_factorzation :2909)
 *   - smoothers: lexicographic SOR       (AMG_SOR_smoother, LinA/Multigrid.c:1345)
 *                damped Jacobi and multicolour SOR (the GPU library's smoothers,
 *                same per-row update as AMG_SOR_smoother)
 *   - pcg                                (LinA/PCGS.c:163-233)
 *   - ILU(0) factors                     (incomplete_LU_factorization,
 *                                          LinA/linear_algebra.c:1952-1982)
 * The hierarchy (level matrices, P, R, labels) is an input.  Parity of this
 * restatement is pinned against the reference's own outputs stored under
 * tests/golden/ (generated by tests/golden/make_golden.py).
 */
#ifndef LINA_PORT_H
#define LINA_PORT_H

#ifdef __cplusplus
extern "C" {
#endif

#define PORT_SMOOTHER_REF_SOR 0
#define PORT_SMOOTHER_JACOBI 2
#define PORT_SMOOTHER_MC_SOR 3

typedef struct port_amg port_amg;

port_amg* port_amg_new(int depth, int smoother, double omega, int nu, int nu_finest);
/* level l: matrix A (n x n); for l > 0 also labels, P (n x nc) and R (nc x n) */
int port_amg_set_level(port_amg* h, int l, int n, const int* A_ptr, const int* A_col, const double* A_val,
                       const int* labels, const int* P_ptr, const int* P_col, const double* P_val,
                       const int* R_ptr, const int* R_col, const double* R_val, int nc);
int port_amg_finalize(port_amg* h);      /* colourings and the coarsest LU */
/* AMG_setup (LinA/Multigrid.c:1613-1754) restated (amg_setup_port.c): builds every level of a handle
   from port_amg_new from the finest matrix (CSR, sorted columns) and finalizes it.  coarsening: 1
   aggressive (finest level only), 2 standard.  0, or a negative code: -1 bad argument, -3 a negative
   diagonal (the restated solve does not apply the reference's row signs), -4 inconsistent coarse
   count, -5 a zero diagonal in the interpolation, -6 an erroneous coarse matrix (the reference aborts
   on the last two), -2 a zero pivot in the coarsest factorisation. */
int port_amg_setup(port_amg* h, int n, const int* ptr, const int* col, const double* val, int dof, int depth,
                   int coarsening, double eps_minus, double eps_plus, double matrix_tol);
/* sizes and host copies of a level (any output pointer may be NULL) */
int port_amg_level_info(const port_amg* h, int l, int* n, long* nnz_A, long* nnz_P, long* nnz_R);
int port_amg_level_export(const port_amg* h, int l, int* labels, int* A_ptr, int* A_col, double* A_val,
                          int* P_ptr, int* P_col, double* P_val, int* R_ptr, int* R_col, double* R_val);
void port_amg_free(port_amg* h);
int port_amg_colouring(const port_amg* h, int l, int* colour);

/* z = M^-1 r: one V-cycle from the zero guess after the isolated-row fix */
void port_vcycle(port_amg* h, const double* r, double* z);
/* pcg with the one-V-cycle preconditioner; returns iterations.  stop_rule 0 is the
   reference's ||r||/||M^-1 r0||, 1 is ||r||/||b||.  max_seconds > 0 bounds the wall time. */
int port_pcg(port_amg* h, const double* b, double* x, double tol, int max_iter, int stop_rule,
             double max_seconds, double* pcg_res);
void port_spmv(const port_amg* h, int l, const double* x, double* y);
/* ILU(0) factors on A's pattern (L_ij where j <= i, U_ij where j > i); 1, or 0 on a zero pivot */
int port_ilu0(int n, const int* ptr, const int* col, const double* a, double* f);
/* BiCGStab_solve (LinA/BiCGStab.c:115-198) on y = A x with the ILU(0) preconditioner of factors f from
   port_ilu0 (use_ilu = 0: none); x holds the start and receives the solution.  Returns the iteration
   count, -1 if memory ran out; *rel_out (if given) = ||R|| / ||R0|| at the end. */
int port_bicgstab_ilu(int n, const int* ptr, const int* col, const double* a, const double* f, const double* b,
                      double* x, double eps, int max_iter, int use_ilu, double* rel_out);

#ifdef __cplusplus
}
#endif

#endif
