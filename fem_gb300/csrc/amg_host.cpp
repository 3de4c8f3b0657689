// amg_host.cpp - AMG setup on the host: strength, C/F splitting, interpolation,
// truncation, Galerkin product and the coarsest-level factorisation.
//
// Each function states the reference routine whose integer and floating-point
// behaviour it reproduces.  Data structures are this library's own (CSR rows,
// a binary heap with lazy deletion instead of a red-black tree); where the
// reference's row-list type has visible side effects (the explicit (i, 0.0)
// entry every new row starts with, the row reset when a last element is
// removed) those effects are reproduced because they decide sparsity patterns.
#include "amg_host.h"

#include <algorithm>
#include <climits>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <queue>

namespace lina {
namespace {

// ------------------------------------------------------------------ rows
struct Row {
    std::vector<int> c;
    std::vector<double> v;
};

// insert_sparse (linear_algebra.c:1124): accumulate into an existing column
// or insert at the sorted position.
inline void row_insert(Row& r, double a, int j) {
    auto it = std::lower_bound(r.c.begin(), r.c.end(), j);
    size_t pos = size_t(it - r.c.begin());
    if (it != r.c.end() && *it == j) {
        r.v[pos] += a;
    } else {
        r.c.insert(it, j);
        r.v.insert(r.v.begin() + pos, a);
    }
}

// remove_element (linear_algebra.c:1181)
inline void row_remove(Row& r, int j) {
    auto it = std::lower_bound(r.c.begin(), r.c.end(), j);
    if (it != r.c.end() && *it == j) {
        size_t pos = size_t(it - r.c.begin());
        r.c.erase(it);
        r.v.erase(r.v.begin() + pos);
    }
}

// delete_zeros (linear_algebra.c:793) on one row whose index is i: rows of
// length > 1 lose their zero entries; a row that would become empty is reset
// to the single entry (i, 0.0) as remove_element_at does (:1161-1178).
inline void row_delete_zeros(std::vector<int>& c, std::vector<double>& v, int i) {
    if (c.size() <= 1) return;
    size_t w = 0;
    for (size_t k = 0; k < c.size(); k++)
        if (v[k] != 0.0) {
            c[w] = c[k];
            v[w] = v[k];
            w++;
        }
    if (w == 0) {
        c.assign(1, i);
        v.assign(1, 0.0);
    } else {
        c.resize(w);
        v.resize(w);
    }
}

inline double csr_diag(const Csr& A, int i) {  // get_diag (linear_algebra.c:3434)
    auto b = A.col.begin() + A.ptr[i], e = A.col.begin() + A.ptr[i + 1];
    auto it = std::lower_bound(b, e, i);
    if (it != e && *it == i) return A.val[size_t(it - A.col.begin())];
    return 0.0;
}

// ------------------------------------------------------------ lists (CSR of ints)
struct Lists {
    std::vector<int> ptr{0};
    std::vector<int> idx;
    int size(int i) const { return ptr[i + 1] - ptr[i]; }
    const int* row(int i) const { return idx.data() + ptr[i]; }
};

// Transpose lists: T[k] lists j in increasing j for every k in S[j]
// (get_strong_connection_sets, Multigrid.c:240-258).
Lists transpose_lists(const Lists& S, int n) {
    Lists T;
    T.ptr.assign(n + 1, 0);
    for (int k : S.idx) T.ptr[k + 1]++;
    for (int i = 0; i < n; i++) T.ptr[i + 1] += T.ptr[i];
    T.idx.resize(S.idx.size());
    std::vector<int> fill(T.ptr.begin(), T.ptr.end() - 1);
    int n_s = (int)S.ptr.size() - 1;
    for (int j = 0; j < n_s; j++)
        for (int p = S.ptr[j]; p < S.ptr[j + 1]; p++) T.idx[fill[S.idx[p]]++] = j;
    return T;
}

// get_max_coupled + get_strong_connected (Multigrid.c:86-97, :156-184):
// j is strong for i when (same unknown and) a_ij < -eps_minus|a_i,min| or
// a_ij > eps_plus|a_i,min|, where a_i,min is the most negative off-diagonal.
Lists strong_connections(const Csr& A, const std::vector<int>& lev, double em, double ep) {
    Lists S;
    S.ptr.resize(A.n + 1);
    S.ptr[0] = 0;
    S.idx.reserve(A.col.size());
    for (int i = 0; i < A.n; i++) {
        double mn = 0.0;
        int mi = -1;
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++)
            if (A.col[p] != i && A.val[p] < mn) {
                mn = A.val[p];
                mi = p;
            }
        if (mi >= 0) {
            double lo = -em * std::fabs(A.val[mi]);
            double hi = ep * std::fabs(A.val[mi]);
            for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                int J = A.col[p];
                if (J == i) continue;
                double a = (lev[i] == lev[J]) ? A.val[p] : 0.0;
                if (a < lo || a > hi) S.idx.push_back(J);
            }
        }
        S.ptr[i + 1] = (int)S.idx.size();
    }
    return S;
}

// Graph view for the coarsener: stored pattern plus "value != 0" flags.
struct Graph {
    int n = 0;
    std::vector<int> ptr, col;
    std::vector<char> nz;
};

Graph graph_of(const Csr& A) {
    Graph g;
    g.n = A.n;
    g.ptr = A.ptr;
    g.col = A.col;
    g.nz.resize(A.val.size());
    for (size_t k = 0; k < A.val.size(); k++) g.nz[k] = (A.val[k] != 0.0);
    return g;
}

// Max-priority queue with the ordering of the reference's red-black tree
// (red_black_tree.c:174-197, :513-523, :620-658): keys compare with '>';
// a new node goes after every node whose key is <= its own, and the largest
// is the rightmost node, so among equal keys the latest insertion wins.  An
// indexed 4-ary heap on (key, insertion sequence) yields the same choice; it
// holds one entry per queued node (a changed key moves the node's entry in
// place), so it never grows past the level's size.
class ImportanceQueue {
   public:
    explicit ImportanceQueue(int n) : pos_(n, -1) {}
    bool contains(int i) const { return pos_[i] >= 0; }
    void insert(int i, double key) {
        if (pos_[i] >= 0) {
            update(i, key);
            return;
        }
        heap_.push_back(Entry{key, ++seq_, i});
        pos_[i] = (int)heap_.size() - 1;
        up(pos_[i]);
    }
    // the node's key changes (and it counts as inserted now)
    void update(int i, double key) {
        const int p = pos_[i];
        const Entry old = heap_[p];
        heap_[p].key = key;
        heap_[p].seq = ++seq_;
        if (before(old, heap_[p]))
            up(p);
        else
            down(p);
    }
    void remove(int i) {
        const int p = pos_[i];
        if (p < 0) return;
        pos_[i] = -1;
        const int last = (int)heap_.size() - 1;
        if (p != last) {
            const Entry moved = heap_[last];
            heap_[p] = moved;
            pos_[moved.node] = p;
            heap_.pop_back();
            up(p);
            down(pos_[moved.node]);
        } else {
            heap_.pop_back();
        }
    }
    int pop_largest() {
        if (heap_.empty()) return -1;
        const int top = heap_[0].node;
        remove(top);
        return top;
    }

   private:
    struct Entry {
        double key;
        uint64_t seq;
        int node;
    };
    // a below b: a smaller key, or an equal key inserted earlier
    static bool before(const Entry& a, const Entry& b) {
        if (a.key > b.key) return false;
        if (b.key > a.key) return true;
        return a.seq < b.seq;
    }
    void up(int p) {
        Entry e = heap_[p];
        while (p > 0) {
            const int q = (p - 1) >> 2;
            if (!before(heap_[q], e)) break;
            heap_[p] = heap_[q];
            pos_[heap_[p].node] = p;
            p = q;
        }
        heap_[p] = e;
        pos_[e.node] = p;
    }
    void down(int p) {
        const int n = (int)heap_.size();
        Entry e = heap_[p];
        for (;;) {
            const int c0 = 4 * p + 1;
            if (c0 >= n) break;
            int c = c0;
            const int ce = std::min(n, c0 + 4);
            for (int k = c0 + 1; k < ce; k++)
                if (before(heap_[c], heap_[k])) c = k;
            if (!before(e, heap_[c])) break;
            heap_[p] = heap_[c];
            pos_[heap_[p].node] = p;
            p = c;
        }
        heap_[p] = e;
        pos_[e.node] = p;
    }
    std::vector<Entry> heap_;
    std::vector<int> pos_;
    uint64_t seq_ = 0;
};

// AMG_coarsener (Multigrid.c:377-473).  `lev` is indexed by the graph's own
// node numbers, exactly as the reference indexes its Levels argument (which,
// in the aggressive second pass, is the fine-level array; the reference's
// behaviour in that case is reproduced, not corrected).
//
// Two pieces of bookkeeping make it fast without changing a label or the
// order of any queue operation:
//  * The importance (AMG_get_lambda, Multigrid.c:364-375) counts, for node J,
//    the undecided and fine nodes of T_J.  Those
//    counts are kept up to date as labels change (a node X changing label
//    touches the J with X in T_J, i.e. J in S_X), so the importance is formed
//    from the same integers without walking T_J.
//  * A node's row is scanned for undecided, not yet queued neighbours.  After
//    one scan every neighbour is queued or decided.  A queued node leaves the
//    queue only when it is decided: a changed key is removed and re-inserted at
//    once.  So a later scan of the same row inserts nothing and is skipped.
void coarsener(const Graph& A, std::vector<int>& label, std::vector<double>& imp, const Lists& S, const Lists& T,
               ImportanceQueue& q, const int* lev, int lev_size, int size, int seed, std::vector<int>& cursor) {
    auto level_of = [&](int i) { return (i < lev_size) ? lev[i] : -1; };
    std::vector<int> undec(size, 0), fine(size, 0);
    for (int j = 0; j < size; j++)
        for (int p = T.ptr[j]; p < T.ptr[j + 1]; p++) {
            const int l = label[T.idx[p]];
            if (l == kUndecided) undec[j]++;
            if (l == kFine) fine[j]++;
        }
    // AMG_get_lambda (Multigrid.c:364-375) from the counts
    auto lambda = [&](int i) { return (double)i / size + undec[i] + 2 * fine[i]; };
    auto decide = [&](int x, int to) {  // label[x]: undecided -> to
        label[x] = to;
        for (int p = S.ptr[x]; p < S.ptr[x + 1]; p++) {
            undec[S.idx[p]]--;
            if (to == kFine) fine[S.idx[p]]++;
        }
    };
    std::vector<char> scanned(size, 0);
    int level = level_of(seed);
    int next = seed;
    do {
        decide(next, kCoarse);
        const int b = A.ptr[next], e = A.ptr[next + 1];
        for (int p = b; p < e; p++) {
            int I = A.col[p];
            if (label[I] == kUndecided && A.nz[p] && !q.contains(I)) q.insert(I, imp[I]);
        }
        for (int p = T.ptr[next]; p < T.ptr[next + 1]; p++) {
            int I = T.idx[p];
            if (q.contains(I)) {
                decide(I, kFine);
                q.remove(I);
            }
        }
        for (int p = b; p < e; p++) {
            int I = A.col[p];
            if (A.nz[p] && q.contains(I)) {
                double lam = lambda(I);
                if (lam != imp[I]) {  // removed and re-inserted: the node's entry moves
                    imp[I] = lam;
                    q.insert(I, lam);
                }
            }
        }
        for (int p = b; p < e; p++) {
            int I = A.col[p];
            if (I == next) continue;
            if (!scanned[I]) {
                for (int r = A.ptr[I]; r < A.ptr[I + 1]; r++) {
                    int J = A.col[r];
                    if (label[J] == kUndecided && A.nz[r] && !q.contains(J)) q.insert(J, imp[J]);
                }
                scanned[I] = 1;
            }
            for (int r = S.ptr[I]; r < S.ptr[I + 1]; r++) {
                int J = S.idx[r];
                if (label[J] == kUndecided) {
                    double lam = lambda(J);
                    if (lam != imp[J]) {  // (re-)inserted with its new key
                        imp[J] = lam;
                        q.insert(J, lam);
                    }
                }
            }
        }
        next = q.pop_largest();
        if (next < 0) {
            // first undecided node of the seed's unknown; labels never return
            // to undecided, so a per-level cursor finds the same node
            int& c = cursor[level + 1];
            while (c < size && !(label[c] == kUndecided && level_of(c) == level)) c++;
            next = (c < size) ? c : -1;
        }
    } while (next >= 0);
}

// AMG_is_isolated (Multigrid.c:498-503)
inline bool is_isolated(const Csr& A, int i) {
    int n = 0;
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++)
        if (A.val[p] != 0.0) n++;
    return n == 1;
}

// standard_coarsening (Multigrid.c:506-548)
int standard_coarsening(const Csr& A, const std::vector<int>& lev, int dof, const Lists& S, const Lists& T,
                        std::vector<int>& label, bool stand_alone) {
    int n = A.n;
    label.assign(n, kUndecided);
    for (int i = 0; i < n; i++) {
        if (S.size(i) == 0) label[i] = is_isolated(A, i) ? kIsolated : kCoarse;
    }
    std::vector<double> imp(n, 0.0);
    ImportanceQueue q(n);
    Graph g = graph_of(A);
    std::vector<int> cursor(dof + 2, 0);
    for (int d = 0; d < dof; d++) {
        int seed = -1;
        for (int j = 0; j < n; j++)
            if (label[j] == kUndecided && lev[j] == d) {
                seed = j;
                break;
            }
        if (seed >= 0) coarsener(g, label, imp, S, T, q, lev.data(), n, n, seed, cursor);
    }
    int coarse = 0;
    for (int i = 0; i < n; i++) {
        if (label[i] == kUndecided) label[i] = kFine;
        if (label[i] == kCoarse) coarse++;
    }
    if (stand_alone)
        for (int i = 0; i < n; i++)
            if (label[i] == kIsolated) coarse++;
    return coarse;
}

// PMIS labels (gpu_pmis.cu) with the reference's handling of points without strong dependencies
// (standard_coarsening, Multigrid.c:506-548: isolated, or coarse) and its count of the coarse
// level (isolated points counted as coarse).  -1 with err set if the device fails.
int pmis_coarsening(const Csr& A, const Lists& S, const Lists& T, std::vector<int>& label, std::string& err) {
    const int n = A.n;
    label.assign(n, kUndecided);
    for (int i = 0; i < n; i++)
        if (S.size(i) == 0) label[i] = is_isolated(A, i) ? kIsolated : kCoarse;
    if (!pmis_gpu(n, S.ptr, S.idx, T.ptr, T.idx, label, err)) return -1;
    int coarse = 0;
    for (int i = 0; i < n; i++)
        if (label[i] == kCoarse || label[i] == kIsolated) coarse++;
    return coarse;
}

// aggressive_coarsening (Multigrid.c:550-607) with Get_2nd_strong_connected
// (:187-217), get_2nd_max_coupled (:99-119) and the distance-two pattern of
// get_2nd_strong_connection_sets (:260-292).
int aggressive_coarsening(const Csr& A, const std::vector<int>& lev, int dof, const Lists& S, const Lists& T,
                          double em, double ep, std::vector<int>& label) {
    int n = A.n;
    std::vector<int> pre;
    int pre_size = standard_coarsening(A, lev, dof, S, T, pre, false);
    label = pre;
    std::vector<int> map(n, -1), inv(pre_size);
    {
        int k = 0;
        for (int i = 0; i < n; i++)
            if (pre[i] == kCoarse) {
                map[i] = k;
                inv[k] = i;
                k++;
            }
    }
    std::vector<double> diag(n);
    for (int i = 0; i < n; i++) diag[i] = csr_diag(A, i);
    Lists M2;
    M2.ptr.assign(pre_size + 1, 0);
    Graph g2;
    g2.n = pre_size;
    g2.ptr.assign(pre_size + 1, 0);
    std::vector<int> cand;
    for (int I = 0; I < pre_size; I++) {
        int i = inv[I];
        double maxv = 0.0;
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int J = A.col[p];
            double val = A.val[p];
            if (J != i && val != 0.0) {
                double d = diag[J];
                for (int r = A.ptr[J]; r < A.ptr[J + 1]; r++) {
                    int K = A.col[r];
                    double val2 = A.val[r];
                    double pv = std::fabs(val * val2 / d);
                    if (K != J && K != i && val2 != 0.0 && pv > maxv) maxv = pv;
                }
            }
        }
        if (maxv > 0.0) {
            double mn = -em * maxv, mx = ep * maxv;
            for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                int J = A.col[p];
                double a = A.val[p];
                double d = diag[J];
                if (J != i && a != 0.0 && lev[i] == lev[J]) {
                    for (int r = A.ptr[J]; r < A.ptr[J + 1]; r++) {
                        int K = A.col[r];
                        double bb = A.val[r];
                        if (pre[K] == kCoarse && K != J && K != i && a * bb / d > 0 && lev[K] == lev[i]) {
                            if (-a * bb / d < mn || a * bb / d > mx) M2.idx.push_back(map[K]);
                        }
                    }
                }
            }
        }
        M2.ptr[I + 1] = (int)M2.idx.size();
        // pattern row I: distinct Map[K] over distance-two coarse neighbours, plus (I, 0.0)
        cand.clear();
        cand.push_back(I);
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int J = A.col[p];
            if (J != i && A.val[p] != 0.0)
                for (int r = A.ptr[J]; r < A.ptr[J + 1]; r++) {
                    int K = A.col[r];
                    if (pre[K] == kCoarse && K != J && K != i && A.val[r] != 0.0) cand.push_back(map[K]);
                }
        }
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        for (int c : cand) {
            g2.col.push_back(c);
            g2.nz.push_back(c != I);
        }
        g2.ptr[I + 1] = (int)g2.col.size();
    }
    Lists T2 = transpose_lists(M2, pre_size);
    std::vector<int> label2(pre_size, kUndecided);
    std::vector<double> imp2(pre_size, 0.0);  // malloc'd without initialisation in the reference
    ImportanceQueue q(pre_size);
    std::vector<int> cursor(dof + 2, 0);
    for (int d = 0; d < dof; d++) {
        int seed = -1;
        for (int I = 0; I < pre_size; I++)
            if (lev[inv[I]] == d) {
                seed = I;
                break;
            }
        if (seed >= 0) coarsener(g2, label2, imp2, M2, T2, q, lev.data(), n, pre_size, seed, cursor);
    }
    int coarse = 0;
    for (int i = 0; i < n; i++) {
        if (label[i] == kCoarse) {
            label[i] = label2[map[i]];
            if (label[i] == kCoarse) coarse++;
        } else if (label[i] == kIsolated) {
            coarse++;
        }
    }
    return coarse;
}

// get_AMG_index_map (Multigrid.c:323-338) with WITH_ISOLATED: every non-fine
// node gets the next coarse index.
int coarse_map(const std::vector<int>& label, std::vector<int>& map) {
    int k = 0;
    map.assign(label.size(), -1);
    for (size_t i = 0; i < label.size(); i++)
        if (label[i] != kFine) map[i] = k++;
    return k;
}

// AMG_simple_standard_interpolation (Multigrid.c:989-1079) followed by
// sparse_approximate (linear_algebra.c:1418-1442) and normalize_row_sum
// (:455-464).  Returns false if a zero diagonal makes the reference abort.
// Sparse accumulator for one row: mark[c] == id means column c is present.
// A removal clears the mark; a later insertion of the same column starts from
// the inserted value, exactly like remove_element followed by insert_sparse.
struct RowAcc {
    std::vector<double> val;
    std::vector<int> mark;
    std::vector<int> touched;
    std::vector<uint64_t> bits;  // touched columns of the row as a bitmap (collect)
    int id = 0, lo = 0, hi = -1;
    explicit RowAcc(int n) : val(n, 0.0), mark(n, -1), bits((size_t)n / 64 + 1, 0) {}
    void begin() {
        id++;
        touched.clear();
        lo = INT_MAX;
        hi = -1;
    }
    void add(int c, double a) {
        if (mark[c] == id) {
            val[c] += a;
        } else {
            mark[c] = id;
            val[c] = a;
            touched.push_back(c);
            lo = std::min(lo, c);
            hi = std::max(hi, c);
        }
    }
    void remove(int c) {
        if (mark[c] == id) mark[c] = -1;
    }
    // present columns in increasing order with their values.  The touched columns are ordered by
    // a bitmap over their span when that is narrow (the usual case: a row's couplings are local),
    // else by sorting.
    void collect(std::vector<int>& cols, std::vector<double>& vals) {
        cols.clear();
        vals.clear();
        if (touched.empty()) return;
        const int w0 = lo >> 6, w1 = hi >> 6;
        if ((long)(w1 - w0 + 1) <= 8L * (long)touched.size()) {
            for (int c : touched) bits[(size_t)c >> 6] |= 1ull << (c & 63);
            for (int w = w0; w <= w1; w++) {
                uint64_t m = bits[(size_t)w];
                bits[(size_t)w] = 0;
                while (m) {
                    const int c = (w << 6) + __builtin_ctzll(m);
                    m &= m - 1;
                    if (mark[c] == id) {
                        cols.push_back(c);
                        vals.push_back(val[c]);
                    }
                }
            }
            return;
        }
        std::sort(touched.begin(), touched.end());
        int prev = -1;
        for (int c : touched) {
            if (c == prev) continue;
            prev = c;
            if (mark[c] == id) {
                cols.push_back(c);
                vals.push_back(val[c]);
            }
        }
    }
};

// AMG_simple_standard_interpolation (Multigrid.c:989-1079) followed by
// sparse_approximate (linear_algebra.c:1418-1442) and normalize_row_sum
// (:455-464).  Rows are independent, so they are built in parallel; the
// reference leaves its row loop at the first fine row without coarse
// neighbours (Multigrid.c:1057-1059), so every row after that one keeps only
// its initial (i, 0.0) entry.  Returns false if a zero diagonal makes the
// reference abort.
bool interpolation(const Csr& A, const std::vector<int>& label, const std::vector<int>& lev,
                   const std::vector<int>& map, int iter, double tol, Csr& P, std::string& err, bool& broke) {
    const int n = A.n;
    std::vector<double> D(n);
    for (int i = 0; i < n; i++) {
        D[i] = csr_diag(A, i);
        if (D[i] == 0.0) {
            char buf[128];
            snprintf(buf, sizeof buf, "diagonal zero at index %d: standard interpolation not possible", i);
            err = buf;
            return false;
        }
    }
    int ncols = 0;
    for (int c : A.col) ncols = std::max(ncols, c + 1);
    ncols = std::max(ncols, n);
    std::vector<std::vector<int>> rc(n);
    std::vector<std::vector<double>> rv(n);
    std::vector<char> fail(n, 0);
#pragma omp parallel
    {
        RowAcc acc(ncols);
        std::vector<int> qc, sc;
        std::vector<double> qv, sv;
#pragma omp for schedule(dynamic, 256)
        for (int i = 0; i < n; i++) {
            std::vector<int>& pc = rc[i];
            std::vector<double>& pv = rv[i];
            pc.assign(1, i);  // sparse_zero: every row starts as (i, 0.0)
            pv.assign(1, 0.0);
            if (label[i] != kFine) {
                Row r{pc, pv};
                row_insert(r, 1.0, map[i]);
                pc.swap(r.c);
                pv.swap(r.v);
                continue;
            }
            qc.assign(A.col.begin() + A.ptr[i], A.col.begin() + A.ptr[i + 1]);
            qv.resize(qc.size());
            for (int p = A.ptr[i], k = 0; p < A.ptr[i + 1]; p++, k++) qv[k] = A.val[p] / D[i];
            for (int pass = 0; pass < iter; pass++) {
                sc = qc;
                sv = qv;
                acc.begin();
                for (size_t k = 0; k < qc.size(); k++) acc.add(qc[k], qv[k]);
                for (size_t j = 0; j < sc.size(); j++) {
                    int J = sc[j];
                    double q = sv[j];
                    if (J != i && label[J] == kFine && q != 0.0) {
                        acc.remove(J);
                        for (int r = A.ptr[J]; r < A.ptr[J + 1]; r++) {
                            int L = A.col[r];
                            double a = A.val[r] / D[J];
                            if (L != J && a != 0.0) acc.add(L, -a * q);
                        }
                    }
                }
                acc.collect(qc, qv);
            }
            // drop couplings to other unknowns (order preserving)
            size_t w = 0;
            for (size_t k = 0; k < qc.size(); k++)
                if (lev[qc[k]] == lev[i]) {
                    qc[w] = qc[k];
                    qv[w] = qv[k];
                    w++;
                }
            qc.resize(w);
            qv.resize(w);
            double s_p = 0, c_p = 0, s_m = 0, c_m = 0;
            double Di = D[i];
            for (size_t k = 0; k < qc.size(); k++) {
                int J = qc[k];
                double q = qv[k];
                if (J != i) {
                    if (q < 0) {
                        s_m += q;
                        if (label[J] == kCoarse) c_m += q;
                    } else {
                        s_p += q;
                        if (label[J] == kCoarse) c_p += q;
                    }
                } else {
                    Di = q;
                }
            }
            double alpha = 0, beta = 0;
            if (c_m != 0) alpha = -s_m / c_m; else Di += s_m;
            if (c_p != 0) beta = -s_p / c_p; else Di += s_p;
            if (alpha == 0 && beta == 0) {
                fail[i] = 1;
                continue;
            }
            alpha /= Di;
            beta /= Di;
            Row r{pc, pv};
            for (size_t k = 0; k < qc.size(); k++) {
                int J = qc[k];
                double q = qv[k];
                if (J != i && label[J] == kCoarse) {
                    if (q < 0 && alpha != 0) row_insert(r, alpha * q, map[J]);
                    if (q > 0 && beta != 0) row_insert(r, beta * q, map[J]);
                }
            }
            pc.swap(r.c);
            pv.swap(r.v);
        }
    }
    broke = false;
    for (int i = 0; i < n; i++) {
        if (broke) {
            rc[i].assign(1, i);
            rv[i].assign(1, 0.0);
        } else if (fail[i]) {
            broke = true;
            rc[i].assign(1, i);
            rv[i].assign(1, 0.0);
        }
    }
    // delete_zeros, sparse_approximate, normalize_row_sum
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        std::vector<int>& c = rc[i];
        std::vector<double>& v = rv[i];
        row_delete_zeros(c, v, i);
        double mx = 0;
        for (size_t k = 0; k < c.size(); k++) {
            double a = std::fabs(v[k]);
            if (c[k] != i && a > mx) mx = a;
        }
        size_t w = 0;
        for (size_t k = 0; k < c.size(); k++) {
            if (c[k] != i && std::fabs(v[k]) < mx * tol) continue;
            c[w] = c[k];
            v[w] = v[k];
            w++;
        }
        c.resize(w);
        v.resize(w);
        double sum = 0;
        for (double x : v) sum += x;
        if (sum != 0)
            for (double& x : v) x *= 1.0 / sum;
    }
    P = Csr();
    P.n = n;
    P.ptr.assign(n + 1, 0);
    for (int i = 0; i < n; i++) P.ptr[i + 1] = P.ptr[i] + (int)rc[i].size();
    P.col.resize(P.ptr[n]);
    P.val.resize(P.ptr[n]);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        std::copy(rc[i].begin(), rc[i].end(), P.col.begin() + P.ptr[i]);
        std::copy(rv[i].begin(), rv[i].end(), P.val.begin() + P.ptr[i]);
    }
    return true;
}

// get_AMG_transposed (Multigrid.c:308-321): nonzero entries of P transposed
// into rows that start as (k, 0.0); no zero deletion afterwards.
Csr amg_transpose(const Csr& P, int nc) {
    Csr R;
    R.n = nc;
    R.ncols = P.n;
    std::vector<int> cnt(nc + 1, 0);
    for (int k = 0; k < nc; k++) cnt[k + 1] = 1;
    for (int i = 0; i < P.n; i++)
        for (int p = P.ptr[i]; p < P.ptr[i + 1]; p++)
            if (P.val[p] != 0.0 && P.col[p] != i) cnt[P.col[p] + 1]++;
    // (an entry whose fine row index equals its coarse column accumulates onto the (k, 0.0) entry)
    R.ptr.assign(nc + 1, 0);
    for (int k = 0; k < nc; k++) R.ptr[k + 1] = R.ptr[k] + cnt[k + 1];
    R.col.assign(R.ptr[nc], 0);
    R.val.assign(R.ptr[nc], 0.0);
    std::vector<int> fill(nc, 0);
    std::vector<char> diag_done(nc, 0);
    // rows are produced in increasing fine index i; the (k, 0.0) entry sits at column k
    for (int i = 0; i < P.n; i++) {
        for (int p = P.ptr[i]; p < P.ptr[i + 1]; p++) {
            double a = P.val[p];
            int k = P.col[p];
            if (a == 0.0) continue;
            int base = R.ptr[k];
            if (!diag_done[k] && k < i) {  // the initial (k, 0.0) precedes column i
                R.col[base + fill[k]] = k;
                R.val[base + fill[k]] = 0.0;
                fill[k]++;
                diag_done[k] = 1;
            }
            if (k == i) {
                R.col[base + fill[k]] = k;
                R.val[base + fill[k]] = 0.0 + a;
                fill[k]++;
                diag_done[k] = 1;
            } else {
                R.col[base + fill[k]] = i;
                R.val[base + fill[k]] = a;
                fill[k]++;
            }
        }
    }
    for (int k = 0; k < nc; k++)
        if (!diag_done[k]) {  // (k, 0.0) is the last entry of row k
            R.col[R.ptr[k] + fill[k]] = k;
            R.val[R.ptr[k] + fill[k]] = 0.0;
            fill[k]++;
        }
    return R;
}

// square_matrix_clean (linear_algebra.c:3100-3120)
bool square_clean(Csr& A) {
    int n = A.n;
    Csr B;
    B.n = n;
    B.ncols = n;
    B.ptr.assign(n + 1, 0);
    B.col.reserve(A.col.size());
    B.val.reserve(A.val.size());
    for (int i = 0; i < n; i++) {
        size_t start = B.col.size();
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int c = A.col[p];
            double v = A.val[p];
            if (c >= n) {
                if (v != 0.0) return false;
                continue;
            }
            if (v == 0.0 && c != i) continue;
            B.col.push_back(c);
            B.val.push_back(v);
        }
        if (B.col.size() == start) {
            B.col.push_back(i);
            B.val.push_back(0.0);
        }
        B.ptr[i + 1] = (int)B.col.size();
    }
    A = std::move(B);
    return true;
}

// sparse_LU_factorization (linear_algebra.c:3040-3062): the rows holding more
// than one nonzero form a dense block factorised without pivoting; the other
// rows are solved by their diagonal.  The block is stored as its inverse so
// that the GPU coarse solve is one dense matrix-vector product.
bool coarse_factor(const Csr& A, CoarseSolver& cs, std::string& err, int device_min_rows) {
    int n = A.n;
    cs = CoarseSolver();
    cs.n = n;
    cs.in_block.assign(n, 0);
    cs.diag_inv.assign(n, 0.0);
    std::vector<int> map(n, -1);
    for (int i = 0; i < n; i++) {
        int cnt = 0;
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++)
            if (A.val[p] != 0.0) cnt++;
        if (cnt > 1) {
            map[i] = (int)cs.block_rows.size();
            cs.block_rows.push_back(i);
            cs.in_block[i] = 1;
        } else {
            double d = csr_diag(A, i);
            cs.diag_inv[i] = 1.0 / d;
        }
    }
    int m = (int)cs.block_rows.size();
    std::vector<double> M((size_t)m * m, 0.0);
    for (int I = 0; I < m; I++) {
        int i = cs.block_rows[I];
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int J = map[A.col[p]];
            if (J >= 0) M[(size_t)I * m + J] = A.val[p];
        }
    }
    if (device_min_rows > 0 && m >= device_min_rows) {  // inverted on the GPU at upload (gpu_coarse.cu)
        cs.inv = std::move(M);
        cs.inverted = false;
        return true;
    }
    // in-place Gauss-Jordan inversion without pivoting (the reference's LU does not pivot)
    std::vector<double>& X = M;
    for (int k = 0; k < m; k++) {
        double piv = X[(size_t)k * m + k];
        if (piv == 0.0) {
            char buf[128];
            snprintf(buf, sizeof buf, "coarsest level: zero pivot at block row %d", k);
            err = buf;
            return false;
        }
        double ip = 1.0 / piv;
        double* rk = &X[(size_t)k * m];
        for (int j = 0; j < m; j++) rk[j] *= ip;
        rk[k] = ip;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < m; i++) {
            if (i == k) continue;
            double* ri = &X[(size_t)i * m];
            double f = ri[k];
            if (f == 0.0) continue;
            ri[k] = 0.0;
            for (int j = 0; j < m; j++) ri[j] -= f * rk[j];
        }
    }
    cs.inv = std::move(X);
    return true;
}

}  // namespace

namespace {
// one Galerkin factor product: on the GPU when asked for (same bits), on the host otherwise or
// when the GPU product fails
Csr galerkin_product(const Csr& A, const Csr& B, bool gpu) {
    if (gpu) {
        Csr C;
        std::string err;
        if (spgemm_gpu(A, B, C, err)) return C;
        fprintf(stderr, "LinA-GB300: Galerkin product on the host (%s)\n", err.c_str());
    }
    return spgemm_ref(A, B);
}
}  // namespace

// sparse_product (linear_algebra.c:186-222): row i of the result starts as
// (i, 0.0); a*b is accumulated per column in the order of A's row entries;
// zero factors are skipped; delete_zeros runs at the end.
Csr spgemm_ref(const Csr& A, const Csr& B) {
    Csr C;
    C.n = A.n;
    C.ncols = B.ncols;
    int width = std::max(B.ncols, A.n) + 1;
    for (int c : B.col) width = std::max(width, c + 1);
    const int n = A.n;
    const int chunk = 4096;
    const int nchunks = (n + chunk - 1) / chunk;
    std::vector<std::vector<int>> ccol(nchunks);
    std::vector<std::vector<double>> cval(nchunks);
    std::vector<std::vector<int>> clen(nchunks);
#pragma omp parallel
    {
        std::vector<double> acc(width, 0.0);
        std::vector<int> mark(width, -1);
        std::vector<int> cols;
        std::vector<double> vals;
#pragma omp for schedule(dynamic, 1)
        for (int ch = 0; ch < nchunks; ch++) {
            const int i0 = ch * chunk, i1 = std::min(n, i0 + chunk);
            for (int i = i0; i < i1; i++) {
                cols.clear();
                mark[i] = i;
                acc[i] = 0.0;
                cols.push_back(i);
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                    double a = A.val[p];
                    if (a == 0.0) continue;
                    int k = A.col[p];
                    for (int r = B.ptr[k]; r < B.ptr[k + 1]; r++) {
                        double b = B.val[r];
                        if (b == 0.0) continue;
                        int j = B.col[r];
                        if (mark[j] != i) {
                            mark[j] = i;
                            acc[j] = a * b;
                            cols.push_back(j);
                        } else {
                            acc[j] += a * b;
                        }
                    }
                }
                std::sort(cols.begin(), cols.end());
                vals.resize(cols.size());
                for (size_t k = 0; k < cols.size(); k++) vals[k] = acc[cols[k]];
                row_delete_zeros(cols, vals, i);
                ccol[ch].insert(ccol[ch].end(), cols.begin(), cols.end());
                cval[ch].insert(cval[ch].end(), vals.begin(), vals.end());
                clen[ch].push_back((int)cols.size());
            }
        }
    }
    C.ptr.assign(n + 1, 0);
    for (int ch = 0, i = 0; ch < nchunks; ch++)
        for (int len : clen[ch]) {
            C.ptr[i + 1] = C.ptr[i] + len;
            i++;
        }
    C.col.resize(C.ptr[n]);
    C.val.resize(C.ptr[n]);
#pragma omp parallel for schedule(static)
    for (int ch = 0; ch < nchunks; ch++) {
        int base = C.ptr[ch * chunk];
        std::copy(ccol[ch].begin(), ccol[ch].end(), C.col.begin() + base);
        std::copy(cval[ch].begin(), cval[ch].end(), C.val.begin() + base);
    }
    return C;
}

int greedy_colouring(const Csr& A, std::vector<int>& colour) {
    int n = A.n;
    std::vector<int> tptr(n + 1, 0);
    for (int i = 0; i < n; i++)
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int j = A.col[p];
            if (j != i && j < n && A.val[p] != 0.0) tptr[j + 1]++;
        }
    for (int i = 0; i < n; i++) tptr[i + 1] += tptr[i];
    std::vector<int> tadj(tptr[n]);
    std::vector<int> fill(tptr.begin(), tptr.end() - 1);
    for (int i = 0; i < n; i++)
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int j = A.col[p];
            if (j != i && j < n && A.val[p] != 0.0) tadj[fill[j]++] = i;
        }
    colour.assign(n, -1);
    std::vector<int> mark(n + 2, -1);
    int ncol = 0;
    for (int i = 0; i < n; i++) {
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int j = A.col[p];
            if (j != i && j < n && A.val[p] != 0.0 && colour[j] >= 0) mark[colour[j]] = i;
        }
        for (int p = tptr[i]; p < tptr[i + 1]; p++)
            if (colour[tadj[p]] >= 0) mark[colour[tadj[p]]] = i;
        int c = 0;
        while (mark[c] == i) c++;
        colour[i] = c;
        ncol = std::max(ncol, c + 1);
    }
    return ncol;
}

bool amg_setup_host(const Csr& Ain, const AmgParams& p, HostHierarchy& h) {
    h = HostHierarchy();
    h.params = p;
    const int depth = p.depth;
    if (depth < 1 || Ain.n <= 0) {
        h.error = "invalid depth or empty matrix";
        return false;
    }
    h.lv.resize(depth);
    // clone + make_positive_diag (linear_algebra.c:2612-2620)
    HostLevel& fine = h.lv[depth - 1];
    fine.A = Ain;
    fine.A.ncols = Ain.n;
    h.signs.assign(Ain.n, 1.0);
    for (int i = 0; i < Ain.n; i++) {
        if (csr_diag(fine.A, i) < 0) {
            for (int q = fine.A.ptr[i]; q < fine.A.ptr[i + 1]; q++) fine.A.val[q] *= -1.0;
            h.signs[i] = -1.0;
        }
    }
    // AMG_init_finest_tupels (Multigrid.c:785-804): block unknown ordering
    {
        int n = Ain.n;
        int mesh = n / p.dof;
        fine.dof_level.assign(n, 0);
        for (int k = 0; k < n; k++) fine.dof_level[k] = (mesh > 0) ? std::min(k / mesh, p.dof - 1) : 0;
    }
    const bool timing = std::getenv("LINA_SETUP_TIMING") != nullptr;
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto secs = [](auto a, auto b) { return std::chrono::duration<double>(b - a).count(); };
    for (int i = depth - 1; i > 0; i--) {
        auto t0 = now();
        HostLevel& L = h.lv[i];
        HostLevel& C = h.lv[i - 1];
        const std::vector<int>& lev = L.dof_level;
        Lists S = strong_connections(L.A, lev, p.eps_minus, p.eps_plus);
        Lists T = transpose_lists(S, L.A.n);
        auto t1 = now();
        bool aggressive = (p.coarsening == kAggressive && i == depth - 1);
        if (aggressive) {
            L.coarse_size = aggressive_coarsening(L.A, lev, p.dof, S, T, p.eps_minus, p.eps_plus, L.labels);
        } else if (p.coarsening == kPmis) {
            L.coarse_size = pmis_coarsening(L.A, S, T, L.labels, h.error);
            if (L.coarse_size < 0) return false;
        } else {
            L.coarse_size = standard_coarsening(L.A, lev, p.dof, S, T, L.labels, true);
        }
        auto t2 = now();
        std::vector<int> map;
        int nc = coarse_map(L.labels, map);
        if (nc != L.coarse_size) {
            h.error = "coarse size disagrees with the number of non-fine labels";
            return false;
        }
        C.dof_level.assign(nc, 0);
        for (int k = 0; k < L.A.n; k++)
            if (map[k] >= 0) C.dof_level[map[k]] = lev[k];
        bool broke = false;
        if (!interpolation(L.A, L.labels, lev, map, aggressive ? 2 : 1, p.matrix_tol, L.P, h.error, broke))
            return false;
        L.P.ncols = nc;
        if (broke) fprintf(stderr, "LinA-GB300 warning: AMG level %d has a fine row without coarse interpolation\n", i);
        auto t3 = now();
        L.R = amg_transpose(L.P, nc);
        Csr AP = galerkin_product(L.A, L.P, p.gpu_products);
        AP.ncols = nc;
        C.A = galerkin_product(L.R, AP, p.gpu_products);
        C.A.ncols = nc;
        if (!square_clean(C.A)) {
            h.error = "erroneous coarse matrix";
            return false;
        }
        auto t4 = now();
        if (timing)
            fprintf(stderr, "level %d n=%d nnz=%lld: strength %.2fs coarsen %.2fs interp %.2fs galerkin %.2fs\n", i,
                    L.A.n, (long long)L.A.nnz(), secs(t0, t1), secs(t1, t2), secs(t2, t3), secs(t3, t4));
    }
    auto tc = now();
    bool ok = coarse_factor(h.lv[0].A, h.coarse, h.error, p.coarse_device_rows);
    if (timing) fprintf(stderr, "coarsest n=%d block=%zu: %.2fs\n", h.lv[0].A.n, h.coarse.block_rows.size(), secs(tc, now()));
    return ok;
}

bool amg_recompute_host(HostHierarchy& h, const Csr& A) {
    const int depth = h.params.depth;
    if ((int)h.lv.size() != depth || A.n != h.lv[depth - 1].A.n) {
        h.error = "matrix size does not match the hierarchy";
        return false;
    }
    h.lv[depth - 1].A = A;
    h.lv[depth - 1].A.ncols = A.n;
    for (int i = depth - 1; i > 0; i--) {
        HostLevel& L = h.lv[i];
        Csr AP = galerkin_product(L.A, L.P, h.params.gpu_products);
        AP.ncols = L.coarse_size;
        h.lv[i - 1].A = galerkin_product(L.R, AP, h.params.gpu_products);
        h.lv[i - 1].A.ncols = L.coarse_size;
        if (!square_clean(h.lv[i - 1].A)) {
            h.error = "erroneous coarse matrix";
            return false;
        }
    }
    return coarse_factor(h.lv[0].A, h.coarse, h.error, h.params.coarse_device_rows);
}

// ---------------------------------------------------------------- hierarchy files
// A matrix file is the reference's write_sparse format (LinA/linear_algebra.c:832-845): int n,
// int Len[n], then every row's column indices, then every row's values (native byte order).

bool write_csr_file(const std::string& path, const Csr& A) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    bool ok = fwrite(&A.n, sizeof(int), 1, f) == 1;
    std::vector<int> len(A.n);
    for (int i = 0; i < A.n; i++) len[i] = A.ptr[i + 1] - A.ptr[i];
    ok = ok && (A.n == 0 || fwrite(len.data(), sizeof(int), A.n, f) == (size_t)A.n);
    ok = ok && (A.col.empty() || fwrite(A.col.data(), sizeof(int), A.col.size(), f) == A.col.size());
    ok = ok && (A.val.empty() || fwrite(A.val.data(), sizeof(double), A.val.size(), f) == A.val.size());
    return fclose(f) == 0 && ok;
}

bool read_csr_file(const std::string& path, Csr& A, int ncols) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    int n = 0;
    bool ok = fread(&n, sizeof(int), 1, f) == 1 && n >= 0;
    std::vector<int> len(ok ? n : 0);
    ok = ok && (n == 0 || fread(len.data(), sizeof(int), n, f) == (size_t)n);
    A = Csr();
    A.n = n;
    A.ncols = ncols;
    A.ptr.assign(n + 1, 0);
    for (int i = 0; ok && i < n; i++) {
        ok = len[i] >= 0 && (long)A.ptr[i] + len[i] <= INT32_MAX;
        if (ok) A.ptr[i + 1] = A.ptr[i] + len[i];
    }
    if (ok) {
        A.col.resize(A.ptr[n]);
        A.val.resize(A.ptr[n]);
        ok = (A.col.empty() || fread(A.col.data(), sizeof(int), A.col.size(), f) == A.col.size()) &&
             (A.val.empty() || fread(A.val.data(), sizeof(double), A.val.size(), f) == A.val.size());
    }
    // columns inside the operand, or the (i, 0.0) placeholder of an empty row
    for (size_t k = 0; ok && k < A.col.size(); k++) ok = A.col[k] >= 0 && A.col[k] < std::max(ncols, n);
    fclose(f);
    return ok;
}

namespace {

bool write_ints(const std::string& path, const std::vector<int>& v) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    const int n = (int)v.size();
    bool ok = fwrite(&n, sizeof(int), 1, f) == 1 && (n == 0 || fwrite(v.data(), sizeof(int), n, f) == (size_t)n);
    return fclose(f) == 0 && ok;
}

bool read_ints(const std::string& path, std::vector<int>& v, int expect) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    int n = 0;
    bool ok = fread(&n, sizeof(int), 1, f) == 1 && n == expect;
    v.assign(ok ? n : 0, 0);
    ok = ok && (n == 0 || fread(v.data(), sizeof(int), n, f) == (size_t)n);
    fclose(f);
    return ok;
}

std::string level_file(const std::string& dir, int l, const char* what) {
    char buf[64];
    snprintf(buf, sizeof buf, "/L%d_%s", l, what);
    return dir + buf;
}

}  // namespace

bool amg_save_host(const HostHierarchy& h, const std::string& dir, std::string& err) {
    const AmgParams& p = h.params;
    FILE* f = fopen((dir + "/hierarchy.txt").c_str(), "w");
    if (!f) {
        err = "cannot write " + dir + "/hierarchy.txt";
        return false;
    }
    // doubles in hexadecimal so that they read back exactly
    fprintf(f, "lina-gb300-amg 1\ndepth %d\ndof %d\ncoarsening %d\nsmoothing %d %d\neps %a %a\nmatrix_tol %a\n"
               "signs %d\n",
            p.depth, p.dof, p.coarsening, p.smoothing_iterations, p.aggr_smoothing_iterations, p.eps_minus,
            p.eps_plus, p.matrix_tol, h.signs.empty() ? 0 : 1);
    for (int l = 0; l < p.depth; l++) fprintf(f, "level %d %d %d\n", l, h.lv[l].A.n, h.lv[l].coarse_size);
    bool ok = fclose(f) == 0;
    for (int l = 0; ok && l < p.depth; l++) {
        const HostLevel& L = h.lv[l];
        ok = write_csr_file(level_file(dir, l, "A"), L.A) && write_ints(level_file(dir, l, "dof_level"), L.dof_level);
        if (ok && l > 0)
            ok = write_csr_file(level_file(dir, l, "P"), L.P) && write_csr_file(level_file(dir, l, "R"), L.R) &&
                 write_ints(level_file(dir, l, "labels"), L.labels);
    }
    if (ok && !h.signs.empty()) {
        FILE* g = fopen((dir + "/signs").c_str(), "wb");
        ok = g && fwrite(h.signs.data(), sizeof(double), h.signs.size(), g) == h.signs.size();
        if (g) ok = (fclose(g) == 0) && ok;
    }
    if (!ok) err = "writing the hierarchy files in " + dir + " failed";
    return ok;
}

bool amg_load_host(const std::string& dir, HostHierarchy& h, int coarse_device_rows) {
    h = HostHierarchy();
    FILE* f = fopen((dir + "/hierarchy.txt").c_str(), "r");
    if (!f) {
        h.error = "cannot read " + dir + "/hierarchy.txt";
        return false;
    }
    AmgParams& p = h.params;
    int version = 0, has_signs = 0;
    bool ok = fscanf(f, " lina-gb300-amg %d depth %d dof %d coarsening %d smoothing %d %d eps %la %la matrix_tol %la "
                        "signs %d",
                     &version, &p.depth, &p.dof, &p.coarsening, &p.smoothing_iterations, &p.aggr_smoothing_iterations,
                     &p.eps_minus, &p.eps_plus, &p.matrix_tol, &has_signs) == 10 &&
              version == 1 && p.depth >= 1 && p.depth <= 64 && p.dof >= 1;
    std::vector<int> sizes, coarse;
    for (int l = 0; ok && l < p.depth; l++) {
        int ll = -1, n = -1, c = -1;
        ok = fscanf(f, " level %d %d %d", &ll, &n, &c) == 3 && ll == l && n >= 0 && c >= 0;
        sizes.push_back(n);
        coarse.push_back(c);
    }
    fclose(f);
    if (ok) h.lv.assign(p.depth, HostLevel());
    for (int l = 0; ok && l < p.depth; l++) {
        HostLevel& L = h.lv[l];
        const int n = sizes[l];
        L.coarse_size = coarse[l];
        ok = read_csr_file(level_file(dir, l, "A"), L.A, n) && L.A.n == n &&
             read_ints(level_file(dir, l, "dof_level"), L.dof_level, n);
        if (ok && l > 0) {
            const int nc = sizes[l - 1];
            ok = read_csr_file(level_file(dir, l, "P"), L.P, nc) && L.P.n == n &&
                 read_csr_file(level_file(dir, l, "R"), L.R, n) && L.R.n == nc &&
                 read_ints(level_file(dir, l, "labels"), L.labels, n);
        }
    }
    if (ok && has_signs) {
        const int n = sizes[p.depth - 1];
        h.signs.assign(n, 0.0);
        FILE* g = fopen((dir + "/signs").c_str(), "rb");
        ok = g && fread(h.signs.data(), sizeof(double), n, g) == (size_t)n;
        if (g) fclose(g);
    }
    if (!ok) {
        h.error = "the hierarchy files in " + dir + " are missing or inconsistent";
        return false;
    }
    h.params.coarse_device_rows = coarse_device_rows;
    return coarse_factor(h.lv[0].A, h.coarse, h.error, coarse_device_rows);
}

}  // namespace lina
