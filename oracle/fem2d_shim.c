/* Test infrastructure (oracle): the reference's P1 stiffness assembly run on a given mesh.
 *
 * FEM2D/FEM2D.c assembles the P1 Laplacian with set_matrix_Aij_11_2D (:5949): per node i the
 * diagonal integral matrix_Aii_11 (:2783, over the fan of triangles around i) and per neighbour j the
 * edge integral matrix_Aij_11 (:2850, over the one or two triangles sharing the edge, found by
 * overlap, :1071), each a 2 x 2 gradient product whose trace insert_A_bbV (:4740) enters as the
 * matrix entry.  The mesh is the reference's global mesh2D: node coordinates, neighbour lists, and the
 * boundary marks and angular neighbour order that the reference's own sort_knots (:1787) computes.
 * Plane-strain elasticity is assembled as crack.c does (Crack/crack.c:10359-10365): lambda times the
 * integrals entered by insert_A_abV_b, plus mu times those of insert_A_baV_b and insert_A_bbV_a
 * (:4716-4733), combined with the reference's scalar_sparse_mult and sparse_add, displacement
 * components blocked (x of node i at i, y at i + n).
 * This file fills that mesh from coordinates and unordered neighbour lists, runs the reference's
 * functions, and returns the matrix as CSR with ascending columns.  Built from the reference's sources
 * where they lie (oracle/Makefile, target fem2d); nothing here is used by the GPU library.
 */
#include <stdlib.h>
#include <string.h>

#include "FEM2D.h"

extern mesh2D glob_mesh;

static long to_csr(sparse_matrix* K, int rows, int* ptr, int* col, double* val, long cap) {
    long nnz = 0;
    for (int i = 0; i < rows; i++) nnz += K->Len[i];
    if (ptr && cap >= nnz) {
        long p = 0;
        ptr[0] = 0;
        for (int i = 0; i < rows; i++) {
            const long r0 = p;
            for (int k = 0; k < K->Len[i]; k++, p++) {
                /* insertion in ascending column order */
                long q = p;
                while (q > r0 && col[q - 1] > K->Indices[i][k]) {
                    col[q] = col[q - 1];
                    val[q] = val[q - 1];
                    q--;
                }
                col[q] = K->Indices[i][k];
                val[q] = K->Values[i][k];
            }
            ptr[i + 1] = (int)p;
        }
    }
    return nnz;
}

/* kind 1: the P1 Laplacian (coefficient 1), n x n; kind 2: plane-strain elasticity with Lame constants
   lambda, mu, 2n x 2n.  Returns the number of stored entries, or -1 when memory runs out.  With
   ptr == NULL (or cap too small) only the count is returned. */
long fs_p1_assemble(int kind, int n, const double* xy, const int* nb_ptr, const int* nb, double lambda, double mu,
                    int* ptr, int* col, double* val, long cap) {
    mesh2D saved = glob_mesh;
    glob_mesh.size = n;
    glob_mesh.Points = (point2D*)malloc((size_t)n * sizeof(point2D));
    glob_mesh.Connections = (int**)calloc((size_t)n, sizeof(int*));
    glob_mesh.Sizes = (int*)malloc((size_t)n * sizeof(int));
    glob_mesh.Is_boundary = (int*)malloc((size_t)n * sizeof(int));
    glob_mesh.Overlap_table = NULL;
    long nnz = -1;
    if (!glob_mesh.Points || !glob_mesh.Connections || !glob_mesh.Sizes || !glob_mesh.Is_boundary) goto done;
    for (int i = 0; i < n; i++) {
        glob_mesh.Points[i].x = xy[2 * i];
        glob_mesh.Points[i].y = xy[2 * i + 1];
        const int len = nb_ptr[i + 1] - nb_ptr[i];
        glob_mesh.Sizes[i] = len;
        glob_mesh.Connections[i] = (int*)malloc((size_t)(len > 0 ? len : 1) * sizeof(int));
        if (!glob_mesh.Connections[i]) goto done;
        memcpy(glob_mesh.Connections[i], nb + nb_ptr[i], (size_t)len * sizeof(int));
    }
    sort_knots();
    if (kind == 1) {
        set_var_number2D(1);
        sparse_matrix* K = set_matrix_Aij_11_2D(0, 0, &insert_A_bbV);
        nnz = to_csr(K, n, ptr, col, val, cap);
        free_sparse(K);
    } else {
        set_var_number2D(2);
        sparse_matrix* K = set_matrix_Aij_11_2D(0, 0, &insert_A_abV_b);
        scalar_sparse_mult(lambda, K);
        sparse_matrix* K2 = set_matrix_Aij_11_2D(0, 0, &insert_A_baV_b);
        sparse_matrix* K3 = set_matrix_Aij_11_2D(0, 0, &insert_A_bbV_a);
        sparse_add(K, K2, mu);
        sparse_add(K, K3, mu);
        nnz = to_csr(K, 2 * n, ptr, col, val, cap);
        free_sparse(K);
        free_sparse(K2);
        free_sparse(K3);
    }
done:
    if (glob_mesh.Connections)
        for (int i = 0; i < n; i++) free(glob_mesh.Connections[i]);
    free(glob_mesh.Points);
    free(glob_mesh.Connections);
    free(glob_mesh.Sizes);
    free(glob_mesh.Is_boundary);
    glob_mesh = saved;
    return nnz;
}
