/*
 * amg_setup_port.c - CPU restatement of the reference's AMG set-up (ORACLE).
 *
 * Test infrastructure and CPU baseline only: the GPU library never links this.
 * It restates AMG_setup (LinA/Multigrid.c:1613-1754) on CSR arrays so that the
 * CPU baseline can build the hierarchy it times without the product library:
 *   - make_positive_diag                    (LinA/linear_algebra.c:2612-2620)
 *   - AMG_init_finest_tupels, AMG_set_tupels (LinA/Multigrid.c:785-830): the
 *     unknown number (Levels) of every row, block ordering on the finest level
 *   - get_max_coupled, get_strong_connected, get_strong_connection_sets
 *                                           (LinA/Multigrid.c:86-97, :156-184, :240-258)
 *   - AMG_get_lambda, AMG_coarsener         (LinA/Multigrid.c:364-473), with the
 *     red-black tree of red_black_tree.c replaced by an indexed binary heap on
 *     (importance, insertion number): the tree places a new key after every
 *     key that is not larger and RBLargest takes the rightmost node, so among
 *     equal importances the latest insertion is taken, which the heap's
 *     insertion number reproduces
 *   - standard_coarsening, aggressive_coarsening with get_2nd_max_coupled,
 *     Get_2nd_strong_connected, get_2nd_strong_connection_sets
 *                                           (LinA/Multigrid.c:506-607, :99-119, :187-217, :260-292)
 *   - get_AMG_index_map (WITH_ISOLATED)     (LinA/Multigrid.c:323-338)
 *   - AMG_simple_standard_interpolation, sparse_approximate, normalize_row_sum
 *                                           (LinA/Multigrid.c:989-1079, :1265-1286;
 *                                            LinA/linear_algebra.c:1418-1442, :455-464)
 *   - get_AMG_transposed                    (LinA/Multigrid.c:308-321)
 *   - get_restricted_matrix: sparse_product twice and square_matrix_clean
 *                                           (LinA/Multigrid.c:475-484;
 *                                            LinA/linear_algebra.c:186-222, :793-806, :3100-3120)
 * The row-list side effects that decide patterns are kept: every new row
 * starts as the single entry (i, 0.0) (sparse_zero), delete_zeros leaves a row
 * whose entries are all zero as (i, 0.0), and the interpolation leaves its row
 * loop at the first fine row without coarse neighbours (Multigrid.c:1057-1059).
 * The reference reads its uninitialised Importance_2nd array in the aggressive
 * second pass (Multigrid.c:566); like the reference run under a zeroing
 * allocator, the array starts at zero here.  Where the reference calls the
 * coarsener with no seed (seed -1, Multigrid.c:574-582) the call is skipped.
 * The coarsest factorisation and the colourings are done by port_amg_finalize
 * (lina_port.c).  Matrices whose set-up flips a row's sign (a negative
 * diagonal) are refused: the restated solve phase does not apply signs.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "lina_port.h"

enum { UNDECIDED = 0, COARSE = 1, FINE = 2, ISOLATED = 3 };
enum { AGGRESSIVE = 1, STANDARD = 2 };

typedef struct {
    int n;      /* rows */
    int ncols;  /* operand size (informational) */
    int* ptr;
    int* col;
    double* val;
} mat_t;

typedef struct { /* lists of ints in CSR form (strong sets) */
    int* ptr;
    int* idx;
} lists_t;

static void mat_free(mat_t* m) {
    free(m->ptr);
    free(m->col);
    free(m->val);
    memset(m, 0, sizeof *m);
}

static void lists_free(lists_t* l) {
    free(l->ptr);
    free(l->idx);
    l->ptr = l->idx = NULL;
}

static double get_diag(const mat_t* A, int i) { /* get_diag, linear_algebra.c:3434 (binary search) */
    int lo = A->ptr[i], hi = A->ptr[i + 1] - 1;
    while (lo <= hi) {
        int mid = (lo + hi) / 2;
        if (A->col[mid] == i) return A->val[mid];
        if (A->col[mid] < i) lo = mid + 1;
        else hi = mid - 1;
    }
    return 0.0;
}

static int cmp_int(const void* a, const void* b) {
    int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

/* ------------------------------------------------------------ growable arrays */
typedef struct {
    int* a;
    long n, cap;
} ivec;
typedef struct {
    double* a;
    long n, cap;
} dvec;

static void ipush(ivec* v, int x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 64;
        v->a = (int*)realloc(v->a, v->cap * sizeof(int));
    }
    v->a[v->n++] = x;
}
static void dpush(dvec* v, double x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 64;
        v->a = (double*)realloc(v->a, v->cap * sizeof(double));
    }
    v->a[v->n++] = x;
}

/* ------------------------------------------------------------ strength */
/* get_strong_connection_sets: S_i lists j in row order, T_k lists i in increasing i */
static void strong_sets(const mat_t* A, const int* lev, double em, double ep, lists_t* S, lists_t* T) {
    const int n = A->n;
    ivec idx = {0};
    S->ptr = (int*)malloc((n + 1) * sizeof(int));
    S->ptr[0] = 0;
    for (int i = 0; i < n; i++) {
        /* get_max_coupled: the most negative off-diagonal entry, first one on ties */
        double mn = 0.0;
        int at = -1;
        for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++)
            if (A->col[p] != i && A->val[p] < mn) {
                mn = A->val[p];
                at = p;
            }
        if (at >= 0) {
            const double lo = -em * fabs(A->val[at]), hi = ep * fabs(A->val[at]);
            for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
                const int j = A->col[p];
                if (j == i) continue;
                const double a = (lev[i] == lev[j]) ? A->val[p] : 0.0;
                if (a < lo || a > hi) ipush(&idx, j);
            }
        }
        S->ptr[i + 1] = (int)idx.n;
    }
    S->idx = idx.a ? idx.a : (int*)malloc(sizeof(int));
    /* transpose */
    T->ptr = (int*)calloc(n + 1, sizeof(int));
    for (long p = 0; p < idx.n; p++) T->ptr[S->idx[p] + 1]++;
    for (int k = 0; k < n; k++) T->ptr[k + 1] += T->ptr[k];
    T->idx = (int*)malloc((idx.n > 0 ? idx.n : 1) * sizeof(int));
    int* fill = (int*)malloc((n + 1) * sizeof(int));
    memcpy(fill, T->ptr, (n + 1) * sizeof(int));
    for (int j = 0; j < n; j++)
        for (int p = S->ptr[j]; p < S->ptr[j + 1]; p++) T->idx[fill[S->idx[p]]++] = j;
    free(fill);
}

/* ------------------------------------------------------------ priority queue */
typedef struct {
    double key;
    uint64_t seq;
    int node;
} hent_t;

typedef struct {
    hent_t* h;
    int n;
    int* pos; /* heap position of each node, -1 when not queued */
    uint64_t seq;
} heap_t;

/* a ranks below b: smaller importance, or the same importance inserted earlier */
static int below(const hent_t* a, const hent_t* b) {
    if (a->key > b->key) return 0;
    if (b->key > a->key) return 1;
    return a->seq < b->seq;
}

static void heap_place(heap_t* q, int p, hent_t e) {
    q->h[p] = e;
    q->pos[e.node] = p;
}

static void sift_up(heap_t* q, int p) {
    hent_t e = q->h[p];
    while (p > 0) {
        int parent = (p - 1) / 2;
        if (!below(&q->h[parent], &e)) break;
        heap_place(q, p, q->h[parent]);
        p = parent;
    }
    heap_place(q, p, e);
}

static void sift_down(heap_t* q, int p) {
    hent_t e = q->h[p];
    for (;;) {
        int c = 2 * p + 1;
        if (c >= q->n) break;
        if (c + 1 < q->n && below(&q->h[c], &q->h[c + 1])) c++;
        if (!below(&e, &q->h[c])) break;
        heap_place(q, p, q->h[c]);
        p = c;
    }
    heap_place(q, p, e);
}

/* RBTreeInsert of a node not in the queue */
static void heap_insert(heap_t* q, int node, double key) {
    hent_t e = {key, ++q->seq, node};
    q->h[q->n] = e;
    q->pos[node] = q->n;
    q->n++;
    sift_up(q, q->n - 1);
}

/* RBDelete */
static void heap_remove(heap_t* q, int node) {
    int p = q->pos[node];
    if (p < 0) return;
    q->pos[node] = -1;
    q->n--;
    if (p == q->n) return;
    const hent_t moved = q->h[q->n];
    heap_place(q, p, moved);
    sift_up(q, p);
    sift_down(q, q->pos[moved.node]);
}

/* RBDelete followed by RBTreeInsert with a new key */
static void heap_reinsert(heap_t* q, int node, double key) {
    heap_remove(q, node);
    heap_insert(q, node, key);
}

/* ------------------------------------------------------------ coarsening */
/* AMG_get_lambda (Multigrid.c:364-375) */
static double get_lambda(const int* label, const lists_t* T, int i, int size) {
    int undec = 0, fine = 0;
    for (int p = T->ptr[i]; p < T->ptr[i + 1]; p++) {
        const int l = label[T->idx[p]];
        if (l == UNDECIDED) undec++;
        if (l == FINE) fine++;
    }
    return (double)i / size + undec + 2 * fine;
}

/* AMG_coarsener (Multigrid.c:377-473).  nz[p] says whether entry p of the graph is nonzero.
   lev is indexed by the graph's own node numbers, as the reference indexes its Levels argument. */
static void coarsener(const int* gptr, const int* gcol, const char* nz, int* label, double* imp,
                      const lists_t* S, const lists_t* T, heap_t* q, const int* lev, int size, int seed) {
    const int level = lev[seed];
    int next = seed;
    /* the reference looks for the first undecided node of the seed's unknown from index 0; labels
       never return to undecided, so a cursor that only moves forward finds the same node */
    int cursor = 0;
    do {
        label[next] = COARSE;
        for (int p = gptr[next]; p < gptr[next + 1]; p++) {
            const int I = gcol[p];
            if (label[I] == UNDECIDED && nz[p] && q->pos[I] < 0) heap_insert(q, I, imp[I]);
        }
        for (int p = T->ptr[next]; p < T->ptr[next + 1]; p++) {
            const int I = T->idx[p];
            if (q->pos[I] >= 0) {
                label[I] = FINE;
                heap_remove(q, I);
            }
        }
        for (int p = gptr[next]; p < gptr[next + 1]; p++) {
            const int I = gcol[p];
            if (nz[p] && q->pos[I] >= 0) {
                const double lam = get_lambda(label, T, I, size);
                if (lam != imp[I]) {
                    imp[I] = lam;
                    heap_reinsert(q, I, lam);
                }
            }
        }
        for (int p = gptr[next]; p < gptr[next + 1]; p++) {
            const int I = gcol[p];
            if (I == next) continue;
            for (int r = gptr[I]; r < gptr[I + 1]; r++) {
                const int J = gcol[r];
                if (label[J] == UNDECIDED && nz[r] && q->pos[J] < 0) heap_insert(q, J, imp[J]);
            }
            for (int r = S->ptr[I]; r < S->ptr[I + 1]; r++) {
                const int J = S->idx[r];
                if (label[J] == UNDECIDED) {
                    const double lam = get_lambda(label, T, J, size);
                    if (lam != imp[J]) {
                        imp[J] = lam;
                        heap_reinsert(q, J, lam);
                    }
                }
            }
        }
        if (q->n > 0) { /* RBLargest */
            next = q->h[0].node;
            heap_remove(q, next);
        } else {
            while (cursor < size && !(label[cursor] == UNDECIDED && lev[cursor] == level)) cursor++;
            next = (cursor < size) ? cursor : -1;
        }
    } while (next >= 0);
}

static int is_isolated(const mat_t* A, int i) { /* AMG_is_isolated, Multigrid.c:498-503 */
    int cnt = 0;
    for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++)
        if (A->val[p] != 0.0) cnt++;
    return cnt == 1;
}

static char* nonzero_flags(const mat_t* A) {
    const long nnz = A->ptr[A->n];
    char* nz = (char*)malloc(nnz > 0 ? nnz : 1);
    for (long p = 0; p < nnz; p++) nz[p] = A->val[p] != 0.0;
    return nz;
}

/* standard_coarsening (Multigrid.c:506-548); stand_alone counts isolated rows as coarse */
static int standard_coarsening(const mat_t* A, const int* lev, int dof, const lists_t* S, const lists_t* T,
                               int* label, int stand_alone) {
    const int n = A->n;
    double* imp = (double*)calloc(n > 0 ? n : 1, sizeof(double));
    heap_t q = {(hent_t*)malloc((n > 0 ? n : 1) * sizeof(hent_t)), 0, (int*)malloc((n > 0 ? n : 1) * sizeof(int)), 0};
    for (int i = 0; i < n; i++) q.pos[i] = -1;
    for (int i = 0; i < n; i++) {
        if (S->ptr[i + 1] == S->ptr[i])
            label[i] = is_isolated(A, i) ? ISOLATED : COARSE;
        else
            label[i] = UNDECIDED;
    }
    char* nz = nonzero_flags(A);
    for (int d = 0; d < dof; d++) {
        int seed = -1;
        for (int j = 0; j < n; j++)
            if (label[j] == UNDECIDED && lev[j] == d) {
                seed = j;
                break;
            }
        if (seed >= 0) coarsener(A->ptr, A->col, nz, label, imp, S, T, &q, lev, n, seed);
    }
    int coarse = 0;
    for (int i = 0; i < n; i++) {
        if (label[i] == UNDECIDED) label[i] = FINE;
        if (label[i] == COARSE) coarse++;
    }
    if (stand_alone)
        for (int i = 0; i < n; i++)
            if (label[i] == ISOLATED) coarse++;
    free(nz);
    free(imp);
    free(q.h);
    free(q.pos);
    return coarse;
}

/* aggressive_coarsening (Multigrid.c:550-607) */
static int aggressive_coarsening(const mat_t* A, const int* lev, int dof, const lists_t* S, const lists_t* T,
                                 double em, double ep, int* label) {
    const int n = A->n;
    int* pre = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
    const int pre_size = standard_coarsening(A, lev, dof, S, T, pre, 0);
    memcpy(label, pre, n * sizeof(int));
    /* get_AMG_index_map without isolated rows */
    int* map = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
    int* inv = (int*)malloc((pre_size > 0 ? pre_size : 1) * sizeof(int));
    for (int i = 0, k = 0; i < n; i++) {
        map[i] = -1;
        if (pre[i] == COARSE) {
            map[i] = k;
            inv[k++] = i;
        }
    }
    double* diag = (double*)malloc((n > 0 ? n : 1) * sizeof(double));
    for (int i = 0; i < n; i++) diag[i] = get_diag(A, i);
    /* Matrix_2nd (strong distance-two sets) and the pattern of Pre_A */
    lists_t M2 = {(int*)calloc(pre_size + 1, sizeof(int)), NULL};
    ivec m2 = {0}, gcol = {0};
    int* gptr = (int*)calloc(pre_size + 1, sizeof(int));
    int* cand = NULL;
    long cand_cap = 0;
    for (int I = 0; I < pre_size; I++) {
        const int i = inv[I];
        /* get_2nd_max_coupled */
        double mx = 0.0;
        for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
            const int J = A->col[p];
            const double val = A->val[p];
            if (J != i && val != 0.0) {
                const double d = diag[J];
                for (int r = A->ptr[J]; r < A->ptr[J + 1]; r++) {
                    const int K = A->col[r];
                    const double val2 = A->val[r];
                    const double pv = fabs(val * val2 / d);
                    if (K != J && K != i && val2 != 0.0 && pv > mx) mx = pv;
                }
            }
        }
        /* Get_2nd_strong_connected */
        if (mx > 0.0) {
            const double lo = -em * mx, hi = ep * mx;
            for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
                const int J = A->col[p];
                const double a = A->val[p];
                const double d = diag[J];
                if (J != i && a != 0.0 && lev[i] == lev[J])
                    for (int r = A->ptr[J]; r < A->ptr[J + 1]; r++) {
                        const int K = A->col[r];
                        const double b = A->val[r];
                        if (pre[K] == COARSE && K != J && K != i && a * b / d > 0 && lev[K] == lev[i])
                            if (-a * b / d < lo || a * b / d > hi) ipush(&m2, map[K]);
                    }
            }
        }
        M2.ptr[I + 1] = (int)m2.n;
        /* row I of Pre_A: (I, 0.0) from sparse_zero, then 1.0 added at Map[K] for every distance-two
           coarse neighbour; only the pattern and which entries are nonzero matter to the coarsener */
        long nc = 0;
        for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
            const int J = A->col[p];
            if (J != i && A->val[p] != 0.0)
                for (int r = A->ptr[J]; r < A->ptr[J + 1]; r++) {
                    const int K = A->col[r];
                    if (pre[K] == COARSE && K != J && K != i && A->val[r] != 0.0) {
                        if (nc + 2 > cand_cap) {
                            cand_cap = cand_cap ? 2 * cand_cap : 256;
                            cand = (int*)realloc(cand, cand_cap * sizeof(int));
                        }
                        cand[nc++] = map[K];
                    }
                }
        }
        if (nc + 1 > cand_cap) {
            cand_cap = cand_cap ? 2 * cand_cap : 256;
            cand = (int*)realloc(cand, cand_cap * sizeof(int));
        }
        cand[nc++] = I;
        qsort(cand, nc, sizeof(int), cmp_int);
        for (long k = 0; k < nc; k++)
            if (k == 0 || cand[k] != cand[k - 1]) ipush(&gcol, cand[k]);
        gptr[I + 1] = (int)gcol.n;
    }
    free(cand);
    M2.idx = m2.a ? m2.a : (int*)malloc(sizeof(int));
    lists_t T2;
    T2.ptr = (int*)calloc(pre_size + 1, sizeof(int));
    for (long p = 0; p < m2.n; p++) T2.ptr[M2.idx[p] + 1]++;
    for (int k = 0; k < pre_size; k++) T2.ptr[k + 1] += T2.ptr[k];
    T2.idx = (int*)malloc((m2.n > 0 ? m2.n : 1) * sizeof(int));
    {
        int* fill = (int*)malloc((pre_size + 1) * sizeof(int));
        memcpy(fill, T2.ptr, (pre_size + 1) * sizeof(int));
        for (int I = 0; I < pre_size; I++)
            for (int p = M2.ptr[I]; p < M2.ptr[I + 1]; p++) T2.idx[fill[M2.idx[p]]++] = I;
        free(fill);
    }
    char* nz2 = (char*)malloc(gcol.n > 0 ? gcol.n : 1);
    for (int I = 0; I < pre_size; I++)
        for (int p = gptr[I]; p < gptr[I + 1]; p++) nz2[p] = gcol.a[p] != I;
    int* label2 = (int*)calloc(pre_size > 0 ? pre_size : 1, sizeof(int)); /* UNDECIDED */
    double* imp2 = (double*)calloc(pre_size > 0 ? pre_size : 1, sizeof(double));
    heap_t q = {(hent_t*)malloc((pre_size > 0 ? pre_size : 1) * sizeof(hent_t)), 0,
                (int*)malloc((pre_size > 0 ? pre_size : 1) * sizeof(int)), 0};
    for (int I = 0; I < pre_size; I++) q.pos[I] = -1;
    for (int d = 0; d < dof; d++) {
        int seed = -1;
        for (int I = 0; I < pre_size; I++)
            if (lev[inv[I]] == d) {
                seed = I;
                break;
            }
        if (seed >= 0) coarsener(gptr, gcol.a, nz2, label2, imp2, &M2, &T2, &q, lev, pre_size, seed);
    }
    int coarse = 0;
    for (int i = 0; i < n; i++) {
        if (label[i] == COARSE) {
            label[i] = label2[map[i]];
            if (label[i] == COARSE) coarse++;
        } else if (label[i] == ISOLATED) {
            coarse++;
        }
    }
    free(pre);
    free(map);
    free(inv);
    free(diag);
    lists_free(&M2);
    lists_free(&T2);
    free(gptr);
    free(gcol.a);
    free(nz2);
    free(label2);
    free(imp2);
    free(q.h);
    free(q.pos);
    return coarse;
}

/* ------------------------------------------------------------ interpolation */
/* one row's sparse accumulator: a removed column is absent until it is inserted again, and then
   starts from the inserted value (remove_element followed by insert_sparse) */
typedef struct {
    double* val;
    int* mark;
    int* touched;
    int nt, cap, id;
} acc_t;

static void acc_init(acc_t* a, int width) {
    a->val = (double*)calloc(width, sizeof(double));
    a->mark = (int*)malloc(width * sizeof(int));
    for (int k = 0; k < width; k++) a->mark[k] = -1;
    a->cap = 256;
    a->touched = (int*)malloc(a->cap * sizeof(int));
    a->nt = 0;
    a->id = 0;
}
static void acc_free(acc_t* a) {
    free(a->val);
    free(a->mark);
    free(a->touched);
}
static void acc_begin(acc_t* a) {
    a->id++;
    a->nt = 0;
}
static void acc_add(acc_t* a, int c, double v) {
    if (a->mark[c] == a->id) {
        a->val[c] += v;
        return;
    }
    a->mark[c] = a->id;
    a->val[c] = v;
    if (a->nt == a->cap) {
        a->cap *= 2;
        a->touched = (int*)realloc(a->touched, a->cap * sizeof(int));
    }
    a->touched[a->nt++] = c;
}
static void acc_remove(acc_t* a, int c) {
    if (a->mark[c] == a->id) a->mark[c] = -1;
}
/* present columns in increasing order */
static void acc_collect(acc_t* a, ivec* cols, dvec* vals) {
    cols->n = vals->n = 0;
    qsort(a->touched, a->nt, sizeof(int), cmp_int);
    for (int k = 0; k < a->nt; k++) {
        const int c = a->touched[k];
        if (k > 0 && c == a->touched[k - 1]) continue;
        if (a->mark[c] == a->id) {
            ipush(cols, c);
            dpush(vals, a->val[c]);
        }
    }
}

/* insert_sparse into a sorted row held in (c, v): accumulate or insert at the sorted place */
static void row_insert(ivec* c, dvec* v, int j, double a) {
    long lo = 0, hi = c->n;
    while (lo < hi) {
        long mid = (lo + hi) / 2;
        if (c->a[mid] < j) lo = mid + 1;
        else hi = mid;
    }
    if (lo < c->n && c->a[lo] == j) {
        v->a[lo] += a;
        return;
    }
    ipush(c, 0);
    dpush(v, 0.0);
    memmove(c->a + lo + 1, c->a + lo, (c->n - 1 - lo) * sizeof(int));
    memmove(v->a + lo + 1, v->a + lo, (v->n - 1 - lo) * sizeof(double));
    c->a[lo] = j;
    v->a[lo] = a;
}

/* delete_zeros (linear_algebra.c:793) on one row with index i */
static void row_delete_zeros(ivec* c, dvec* v, int i) {
    if (c->n <= 1) return;
    long w = 0;
    for (long k = 0; k < c->n; k++)
        if (v->a[k] != 0.0) {
            c->a[w] = c->a[k];
            v->a[w] = v->a[k];
            w++;
        }
    if (w == 0) {
        c->a[0] = i;
        v->a[0] = 0.0;
        w = 1;
    }
    c->n = v->n = w;
}

/* set_prolongation_map (Multigrid.c:1265-1286): AMG_simple_standard_interpolation with `iter`
   elimination passes, sparse_approximate(P, tol), normalize_row_sum(P).  Returns 0, or -1 on a zero
   diagonal (where the reference aborts). */
static int interpolation(const mat_t* A, const int* label, const int* lev, const int* map, int iter, double tol,
                         mat_t* P) {
    const int n = A->n;
    double* D = (double*)malloc((n > 0 ? n : 1) * sizeof(double));
    for (int i = 0; i < n; i++) {
        D[i] = get_diag(A, i);
        if (D[i] == 0.0) {
            free(D);
            return -1;
        }
    }
    int width = n;
    for (long p = 0; p < A->ptr[n]; p++)
        if (A->col[p] + 1 > width) width = A->col[p] + 1;
    ivec* rc = (ivec*)calloc(n > 0 ? n : 1, sizeof(ivec));
    dvec* rv = (dvec*)calloc(n > 0 ? n : 1, sizeof(dvec));
    char* fail = (char*)calloc(n > 0 ? n : 1, 1);
#pragma omp parallel
    {
        acc_t acc;
        acc_init(&acc, width);
        ivec qc = {0}, sc = {0};
        dvec qv = {0}, sv = {0};
#pragma omp for schedule(dynamic, 256)
        for (int i = 0; i < n; i++) {
            ivec* pc = &rc[i];
            dvec* pv = &rv[i];
            ipush(pc, i); /* sparse_zero */
            dpush(pv, 0.0);
            if (label[i] != FINE) {
                row_insert(pc, pv, map[i], 1.0);
                continue;
            }
            /* Q = clone(A) scaled by 1/D[i] */
            qc.n = qv.n = 0;
            for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
                ipush(&qc, A->col[p]);
                dpush(&qv, A->val[p] / D[i]);
            }
            for (int pass = 0; pass < iter; pass++) {
                sc.n = sv.n = 0;
                for (long k = 0; k < qc.n; k++) {
                    ipush(&sc, qc.a[k]);
                    dpush(&sv, qv.a[k]);
                }
                acc_begin(&acc);
                for (long k = 0; k < qc.n; k++) acc_add(&acc, qc.a[k], qv.a[k]);
                for (long k = 0; k < sc.n; k++) {
                    const int J = sc.a[k];
                    const double q = sv.a[k];
                    if (J != i && label[J] == FINE && q != 0.0) {
                        acc_remove(&acc, J);
                        for (int r = A->ptr[J]; r < A->ptr[J + 1]; r++) {
                            const int L = A->col[r];
                            const double a = A->val[r] / D[J];
                            if (L != J && a != 0.0) acc_add(&acc, L, -a * q);
                        }
                    }
                }
                acc_collect(&acc, &qc, &qv);
            }
            /* couplings to other unknowns are dropped, order kept */
            long w = 0;
            for (long k = 0; k < qc.n; k++)
                if (lev[qc.a[k]] == lev[i]) {
                    qc.a[w] = qc.a[k];
                    qv.a[w] = qv.a[k];
                    w++;
                }
            qc.n = qv.n = w;
            double s_p = 0, c_p = 0, s_m = 0, c_m = 0, Di = D[i];
            for (long k = 0; k < qc.n; k++) {
                const int J = qc.a[k];
                const double q = qv.a[k];
                if (J != i) {
                    if (q < 0) {
                        s_m += q;
                        if (label[J] == COARSE) c_m += q;
                    } else {
                        s_p += q;
                        if (label[J] == COARSE) c_p += q;
                    }
                } else {
                    Di = q;
                }
            }
            double alpha = 0, beta = 0;
            if (c_m != 0) alpha = -s_m / c_m;
            else Di += s_m;
            if (c_p != 0) beta = -s_p / c_p;
            else Di += s_p;
            if (alpha == 0 && beta == 0) {
                fail[i] = 1;
                continue;
            }
            alpha /= Di;
            beta /= Di;
            for (long k = 0; k < qc.n; k++) {
                const int J = qc.a[k];
                const double q = qv.a[k];
                if (J != i && label[J] == COARSE) {
                    if (q < 0 && alpha != 0) row_insert(pc, pv, map[J], alpha * q);
                    if (q > 0 && beta != 0) row_insert(pc, pv, map[J], beta * q);
                }
            }
        }
        acc_free(&acc);
        free(qc.a);
        free(sc.a);
        free(qv.a);
        free(sv.a);
    }
    /* the reference's row loop ends at the first fine row without coarse neighbours */
    int broke = 0;
    for (int i = 0; i < n; i++) {
        if (broke || fail[i]) {
            broke = 1;
            rc[i].n = rv[i].n = 1;
            rc[i].a[0] = i;
            rv[i].a[0] = 0.0;
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        ivec* c = &rc[i];
        dvec* v = &rv[i];
        row_delete_zeros(c, v, i);
        double mx = 0;
        for (long k = 0; k < c->n; k++)
            if (c->a[k] != i && fabs(v->a[k]) > mx) mx = fabs(v->a[k]);
        long w = 0;
        for (long k = 0; k < c->n; k++) {
            if (c->a[k] != i && fabs(v->a[k]) < mx * tol) continue;
            c->a[w] = c->a[k];
            v->a[w] = v->a[k];
            w++;
        }
        c->n = v->n = w;
        double sum = 0;
        for (long k = 0; k < v->n; k++) sum += v->a[k];
        if (sum != 0)
            for (long k = 0; k < v->n; k++) v->a[k] *= 1.0 / sum;
    }
    P->n = n;
    P->ptr = (int*)malloc((n + 1) * sizeof(int));
    P->ptr[0] = 0;
    for (int i = 0; i < n; i++) P->ptr[i + 1] = P->ptr[i] + (int)rc[i].n;
    P->col = (int*)malloc((P->ptr[n] > 0 ? P->ptr[n] : 1) * sizeof(int));
    P->val = (double*)malloc((P->ptr[n] > 0 ? P->ptr[n] : 1) * sizeof(double));
    for (int i = 0; i < n; i++) {
        memcpy(P->col + P->ptr[i], rc[i].a, rc[i].n * sizeof(int));
        memcpy(P->val + P->ptr[i], rv[i].a, rv[i].n * sizeof(double));
        free(rc[i].a);
        free(rv[i].a);
    }
    free(rc);
    free(rv);
    free(fail);
    free(D);
    return 0;
}

/* get_AMG_transposed (Multigrid.c:308-321): R = sparse_zero(nc), then every nonzero P_ik inserted at
   (k, i), so row k holds (k, 0.0) (plus P_kk when that is nonzero) and the fine rows i, sorted */
static void amg_transpose(const mat_t* P, int nc, mat_t* R) {
    const int n = P->n;
    int* cnt = (int*)calloc(nc + 1, sizeof(int));
    for (int k = 0; k < nc; k++) cnt[k + 1] = 1;
    for (int i = 0; i < n; i++)
        for (int p = P->ptr[i]; p < P->ptr[i + 1]; p++)
            if (P->val[p] != 0.0 && P->col[p] != i) cnt[P->col[p] + 1]++;
    R->n = nc;
    R->ncols = n;
    R->ptr = (int*)malloc((nc + 1) * sizeof(int));
    R->ptr[0] = 0;
    for (int k = 0; k < nc; k++) R->ptr[k + 1] = R->ptr[k] + cnt[k + 1];
    R->col = (int*)malloc((R->ptr[nc] > 0 ? R->ptr[nc] : 1) * sizeof(int));
    R->val = (double*)malloc((R->ptr[nc] > 0 ? R->ptr[nc] : 1) * sizeof(double));
    int* fill = (int*)calloc(nc > 0 ? nc : 1, sizeof(int));
    char* placed = (char*)calloc(nc > 0 ? nc : 1, 1); /* the (k, 0.0) entry is in place */
    for (int i = 0; i < n; i++)
        for (int p = P->ptr[i]; p < P->ptr[i + 1]; p++) {
            const double a = P->val[p];
            const int k = P->col[p];
            if (a == 0.0) continue;
            const int base = R->ptr[k];
            if (!placed[k] && k < i) {
                R->col[base + fill[k]] = k;
                R->val[base + fill[k]] = 0.0;
                fill[k]++;
                placed[k] = 1;
            }
            if (k == i) {
                R->col[base + fill[k]] = k;
                R->val[base + fill[k]] = 0.0 + a;
                placed[k] = 1;
            } else {
                R->col[base + fill[k]] = i;
                R->val[base + fill[k]] = a;
            }
            fill[k]++;
        }
    for (int k = 0; k < nc; k++)
        if (!placed[k]) {
            R->col[R->ptr[k] + fill[k]] = k;
            R->val[R->ptr[k] + fill[k]] = 0.0;
        }
    free(cnt);
    free(fill);
    free(placed);
}

/* sparse_product (linear_algebra.c:186-222): row i starts as (i, 0.0); products of nonzero factors
   accumulate per column in A's and then B's stored order; delete_zeros at the end */
static void sparse_product(const mat_t* A, const mat_t* B, mat_t* C) {
    const int n = A->n;
    int width = n > B->ncols ? n : B->ncols;
    for (long p = 0; p < B->ptr[B->n]; p++)
        if (B->col[p] + 1 > width) width = B->col[p] + 1;
    const int chunk = 2048;
    const int nchunks = (n + chunk - 1) / chunk;
    ivec* cc = (ivec*)calloc(nchunks > 0 ? nchunks : 1, sizeof(ivec));
    dvec* cv = (dvec*)calloc(nchunks > 0 ? nchunks : 1, sizeof(dvec));
    int* len = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
#pragma omp parallel
    {
        acc_t acc;
        acc_init(&acc, width);
        ivec rcol = {0};
        dvec rval = {0};
#pragma omp for schedule(dynamic, 1)
        for (int ch = 0; ch < nchunks; ch++) {
            const int i0 = ch * chunk, i1 = (i0 + chunk < n) ? i0 + chunk : n;
            for (int i = i0; i < i1; i++) {
                acc_begin(&acc);
                acc_add(&acc, i, 0.0);
                for (int p = A->ptr[i]; p < A->ptr[i + 1]; p++) {
                    const double a = A->val[p];
                    if (a == 0.0) continue;
                    const int k = A->col[p];
                    for (int r = B->ptr[k]; r < B->ptr[k + 1]; r++) {
                        const double b = B->val[r];
                        if (b != 0.0) acc_add(&acc, B->col[r], a * b);
                    }
                }
                acc_collect(&acc, &rcol, &rval);
                row_delete_zeros(&rcol, &rval, i);
                for (long k = 0; k < rcol.n; k++) {
                    ipush(&cc[ch], rcol.a[k]);
                    dpush(&cv[ch], rval.a[k]);
                }
                len[i] = (int)rcol.n;
            }
        }
        acc_free(&acc);
        free(rcol.a);
        free(rval.a);
    }
    C->n = n;
    C->ncols = B->ncols;
    C->ptr = (int*)malloc((n + 1) * sizeof(int));
    C->ptr[0] = 0;
    for (int i = 0; i < n; i++) C->ptr[i + 1] = C->ptr[i] + len[i];
    C->col = (int*)malloc((C->ptr[n] > 0 ? C->ptr[n] : 1) * sizeof(int));
    C->val = (double*)malloc((C->ptr[n] > 0 ? C->ptr[n] : 1) * sizeof(double));
    for (int ch = 0; ch < nchunks; ch++) {
        const int base = C->ptr[ch * chunk];
        memcpy(C->col + base, cc[ch].a, cc[ch].n * sizeof(int));
        memcpy(C->val + base, cv[ch].a, cv[ch].n * sizeof(double));
        free(cc[ch].a);
        free(cv[ch].a);
    }
    free(cc);
    free(cv);
    free(len);
}

/* square_matrix_clean (linear_algebra.c:3100-3120): drops columns >= n (they must be zero) and zero
   off-diagonal entries; a row left empty becomes (i, 0.0).  Returns 0 on a nonzero column >= n. */
static int square_clean(mat_t* A) {
    const int n = A->n;
    long w = 0;
    int start = 0;
    for (int i = 0; i < n; i++) {
        const long row0 = w;
        for (int p = start; p < A->ptr[i + 1]; p++) {
            const int c = A->col[p];
            const double v = A->val[p];
            if (c >= n) {
                if (v != 0.0) return 0;
                continue;
            }
            if (v == 0.0 && c != i) continue;
            A->col[w] = c;
            A->val[w] = v;
            w++;
        }
        if (w == row0) {
            A->col[w] = i;
            A->val[w] = 0.0;
            w++;
        }
        start = A->ptr[i + 1];
        A->ptr[i + 1] = (int)w;
    }
    A->ncols = n;
    return 1;
}

/* ------------------------------------------------------------ AMG_setup */
int port_amg_setup(port_amg* h, int n, const int* ptr, const int* col, const double* val, int dof, int depth,
                   int coarsening, double eps_minus, double eps_plus, double matrix_tol) {
    if (!h || n <= 0 || dof < 1 || depth < 1 || (coarsening != AGGRESSIVE && coarsening != STANDARD)) return -1;
    mat_t A = {n, n, NULL, NULL, NULL};
    A.ptr = (int*)malloc((n + 1) * sizeof(int));
    memcpy(A.ptr, ptr, (n + 1) * sizeof(int));
    A.col = (int*)malloc((ptr[n] > 0 ? ptr[n] : 1) * sizeof(int));
    A.val = (double*)malloc((ptr[n] > 0 ? ptr[n] : 1) * sizeof(double));
    memcpy(A.col, col, ptr[n] * sizeof(int));
    memcpy(A.val, val, ptr[n] * sizeof(double));
    for (int i = 0; i < n; i++)
        if (get_diag(&A, i) < 0) { /* make_positive_diag would flip this row */
            mat_free(&A);
            return -3;
        }
    /* AMG_init_finest_tupels: rows beyond dof * (n / dof) keep the zeroed allocation's 0 */
    int* lev = (int*)calloc(n, sizeof(int));
    const int mesh = n / dof;
    for (int i = 0; i < mesh; i++)
        for (int j = 0; j < dof; j++) lev[j * mesh + i] = j;
    int rc = 0;
    for (int l = depth - 1; l > 0 && rc == 0; l--) {
        lists_t S, T;
        strong_sets(&A, lev, eps_minus, eps_plus, &S, &T);
        int* label = (int*)malloc(A.n * sizeof(int));
        const int aggressive = (coarsening == AGGRESSIVE && l == depth - 1);
        const int nc = aggressive ? aggressive_coarsening(&A, lev, dof, &S, &T, eps_minus, eps_plus, label)
                                  : standard_coarsening(&A, lev, dof, &S, &T, label, 1);
        lists_free(&S);
        lists_free(&T);
        int* map = (int*)malloc(A.n * sizeof(int));
        int k = 0;
        for (int i = 0; i < A.n; i++) map[i] = (label[i] != FINE) ? k++ : -1;
        if (k != nc) rc = -4;
        int* clev = (int*)calloc(nc > 0 ? nc : 1, sizeof(int));
        for (int i = 0; i < A.n; i++)
            if (map[i] >= 0) clev[map[i]] = lev[i];
        mat_t P = {0}, R = {0}, AP = {0}, Ac = {0};
        if (rc == 0 && interpolation(&A, label, lev, map, aggressive ? 2 : 1, matrix_tol, &P) != 0) rc = -5;
        if (rc == 0) {
            P.ncols = nc;
            amg_transpose(&P, nc, &R);
            sparse_product(&A, &P, &AP);
            AP.ncols = nc;
            sparse_product(&R, &AP, &Ac);
            mat_free(&AP);
            if (!square_clean(&Ac)) rc = -6;
        }
        if (rc == 0)
            rc = port_amg_set_level(h, l, A.n, A.ptr, A.col, A.val, label, P.ptr, P.col, P.val, R.ptr, R.col,
                                    R.val, nc);
        mat_free(&P);
        mat_free(&R);
        mat_free(&A);
        free(label);
        free(map);
        free(lev);
        lev = clev;
        A = Ac;
    }
    if (rc == 0) rc = port_amg_set_level(h, 0, A.n, A.ptr, A.col, A.val, NULL, NULL, NULL, NULL, NULL, NULL, NULL, 0);
    mat_free(&A);
    free(lev);
    if (rc == 0) rc = port_amg_finalize(h);
    return rc;
}
