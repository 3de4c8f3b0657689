// gpu_elastic.cu - adjoint gradient of P1 plane-strain elasticity with a
// per-element Young's modulus: GPU assembly of A(E) into a fixed CSR pattern,
// forward AMG-PCG solve with a sensor loss, transposed solve with the same
// hierarchy, and the per-element gradient dL/dE_e = -lambda_e^T Khat_e u_e.
//
// The element arithmetic is the P1 stiffness the reference assembles in
// FEM2D (FEM2D/FEM2D.c:2783-2888, plane strain): with the triangle's
// coefficient vectors b_k = y_{k+1} - y_{k+2}, c_k = x_{k+2} - x_{k+1} and area
// |T|, the strain of a nodal field v is eps(v) = sum_k (b_k vx_k, c_k vy_k,
// c_k vx_k + b_k vy_k) / (2|T|) and K_e = |T| B^T D B with the plane-strain
// elasticity matrix D.  Dirichlet dofs are eliminated symmetrically (identity
// rows, known values lifted into b), which keeps A symmetric.
//
// Assembly is a gather, not a scatter: every stored entry owns the list of
// (element, unit-modulus coefficient) pairs that add into it, in element
// order, so A_p = sum E_e c_e is summed in a fixed order with explicitly
// rounded products and sums (bit-identical to the host assembly, no atomics).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lina_gpu.h"

namespace lina {
namespace dev {
void set_error(const char* msg);
}
}  // namespace lina

namespace {

constexpr int kT = 256;

void fail(const char* fmt, const char* a = "") {
    char buf[512];
    snprintf(buf, sizeof buf, fmt, a);
    lina::dev::set_error(buf);
}

int grid(long n) {
    long g = (n + kT - 1) / kT;
    return (int)std::max(1L, std::min(g, 152L * 16));
}

// ---------------------------------------------------------------- host element arithmetic
struct Geo {
    double beta[3], gamma[3], area;  // b_k/(2|T|), c_k/(2|T|), |T|
};

Geo geometry(const double* xy, const int* t) {
    const double x0 = xy[2 * t[0]], y0 = xy[2 * t[0] + 1];
    const double x1 = xy[2 * t[1]], y1 = xy[2 * t[1] + 1];
    const double x2 = xy[2 * t[2]], y2 = xy[2 * t[2] + 1];
    const double b[3] = {y1 - y2, y2 - y0, y0 - y1};
    const double c[3] = {x2 - x1, x0 - x2, x1 - x0};
    const double area2 = x0 * (y1 - y2) + x1 * (y2 - y0) + x2 * (y0 - y1);
    Geo g;
    g.area = std::fabs(area2) / 2.0;
    const double s = 1.0 / (2.0 * g.area);
    for (int k = 0; k < 3; k++) {
        g.beta[k] = b[k] * s;
        g.gamma[k] = c[k] * s;
    }
    return g;
}

struct Dmat {
    double d00, d01, d11, d22;
};

Dmat plane_strain(double nu) {
    const double f = 1.0 / ((1.0 + nu) * (1.0 - 2.0 * nu));
    return {f * (1.0 - nu), f * nu, f * (1.0 - nu), f * (1.0 - 2.0 * nu) / 2.0};
}

// unit-modulus element stiffness entry for (node a, component p) x (node b, component q)
double khat(const Geo& g, const Dmat& D, int a, int p, int b, int q) {
    const double ba = g.beta[a], ga = g.gamma[a], bb = g.beta[b], gb = g.gamma[b];
    double v;
    if (p == 0 && q == 0)
        v = ba * D.d00 * bb + ga * D.d22 * gb;
    else if (p == 0 && q == 1)
        v = ba * D.d01 * gb + ga * D.d22 * bb;
    else if (p == 1 && q == 0)
        v = ga * D.d01 * bb + ba * D.d22 * gb;
    else
        v = ga * D.d11 * gb + ba * D.d22 * bb;
    return g.area * v;
}

// the assembled structure of a problem: CSR pattern and the contribution lists
struct Plan {
    int nn = 0, ne = 0, n = 0;
    std::vector<int> ptr, col;
    std::vector<int> cptr, celem;  // per stored entry: contributions [cptr[p], cptr[p+1])
    std::vector<double> ccoef;     // celem -1: constant coefficient (identity rows)
    std::vector<int> lptr, lelem;  // per row: lifted Dirichlet contributions to b
    std::vector<double> lcoef;     // unit-modulus coefficient times the known value
    std::vector<unsigned char> fixed;
    std::vector<double> fixval;
    std::vector<double> geo;  // 7 per element: beta[3], gamma[3], area
    Dmat D{};
    int kind = LINA_P1_ELASTIC;  // LINA_P1_LAPLACE: one unknown per node
    int ncomp = 2;
    std::string error;
};

// a P1 mesh with Dirichlet dofs (dof c * n_nodes + node for component c)
struct Mesh {
    int kind = LINA_P1_ELASTIC;
    int nn = 0, ne = 0;
    const double* xy = nullptr;
    const int* tri = nullptr;
    double nu = 0.0;
    int n_fixed = 0;
    const int* fixed_dof = nullptr;
    const double* fixed_val = nullptr;
};

bool check_mesh(const Mesh& m, std::string& err) {
    if ((m.kind != LINA_P1_LAPLACE && m.kind != LINA_P1_ELASTIC) || m.nn <= 0 || m.ne <= 0 || !m.xy || !m.tri ||
        m.n_fixed < 0 || (m.n_fixed > 0 && (!m.fixed_dof || !m.fixed_val))) {
        err = "invalid problem description";
        return false;
    }
    if (m.kind == LINA_P1_ELASTIC && !(m.nu > -1.0 && m.nu < 0.5)) {
        err = "Poisson's ratio outside (-1, 0.5)";
        return false;
    }
    const int nc = m.kind == LINA_P1_ELASTIC ? 2 : 1;
    if ((long)m.nn * nc > (long)INT32_MAX / 8) {
        err = "too many nodes for 32-bit indices";
        return false;
    }
    for (long k = 0; k < 3L * m.ne; k++)
        if (m.tri[k] < 0 || m.tri[k] >= m.nn) {
            err = "triangle node index out of range";
            return false;
        }
    const int n = nc * m.nn;
    std::vector<unsigned char> seen(n, 0);
    for (int k = 0; k < m.n_fixed; k++) {
        const int d = m.fixed_dof[k];
        if (d < 0 || d >= n || seen[d]) {
            err = "Dirichlet dofs out of range or repeated";
            return false;
        }
        seen[d] = 1;
    }
    return true;
}

Mesh mesh_of(const lina_gpu_elastic_problem* p) {
    Mesh m;
    m.kind = LINA_P1_ELASTIC;
    m.nn = p->n_nodes;
    m.ne = p->n_elems;
    m.xy = p->xy;
    m.tri = p->tri;
    m.nu = p->nu;
    m.n_fixed = p->n_fixed;
    m.fixed_dof = p->fixed_dof;
    m.fixed_val = p->fixed_val;
    return m;
}

bool check_problem(const lina_gpu_elastic_problem* p, std::string& err) {
    if (!p || p->n_sensors < 0 || (p->n_sensors > 0 && (!p->sensor_dof || !p->target))) {
        err = "invalid problem description";
        return false;
    }
    if (!check_mesh(mesh_of(p), err)) return false;
    const int n = 2 * p->n_nodes;
    std::vector<unsigned char> fixed(n, 0), sens(n, 0);
    for (int k = 0; k < p->n_fixed; k++) fixed[p->fixed_dof[k]] = 1;
    for (int k = 0; k < p->n_sensors; k++) {
        const int d = p->sensor_dof[k];
        if (d < 0 || d >= n || fixed[d] || sens[d]) {
            err = "sensor dofs out of range, repeated or on a Dirichlet dof";
            return false;
        }
        sens[d] = 1;
    }
    return true;
}

// The CSR pattern of the assembled matrix and, for every stored entry, the (element,
// unit-coefficient value) pairs adding into it in element order; the entry of an element matrix is
// the P1 Laplacian's |T| (beta_a beta_b + gamma_a gamma_b), or the plane-strain stiffness of unit
// modulus (khat).
bool build_plan(const Mesh& mesh, Plan& P) {
    if (!check_mesh(mesh, P.error)) return false;
    const Mesh* p = &mesh;
    const int nc = mesh.kind == LINA_P1_ELASTIC ? 2 : 1;
    const int nn = mesh.nn, ne = mesh.ne, n = nc * nn;
    P.kind = mesh.kind;
    P.ncomp = nc;
    P.nn = nn, P.ne = ne, P.n = n;
    if (mesh.kind == LINA_P1_ELASTIC) P.D = plane_strain(mesh.nu);
    P.fixed.assign(n, 0);
    P.fixval.assign(n, 0.0);
    for (int k = 0; k < p->n_fixed; k++) {
        P.fixed[p->fixed_dof[k]] = 1;
        P.fixval[p->fixed_dof[k]] = p->fixed_val[k];
    }
    // geometry
    P.geo.resize(7L * ne);
    for (int e = 0; e < ne; e++) {
        Geo g = geometry(p->xy, p->tri + 3L * e);
        if (!(g.area > 0.0)) {
            P.error = "degenerate triangle";
            return false;
        }
        for (int k = 0; k < 3; k++) {
            P.geo[7L * e + k] = g.beta[k];
            P.geo[7L * e + 3 + k] = g.gamma[k];
        }
        P.geo[7L * e + 6] = g.area;
    }
    // node adjacency (sorted, including the node itself)
    std::vector<int> deg(nn + 1, 0);
    for (int e = 0; e < ne; e++)
        for (int a = 0; a < 3; a++) deg[p->tri[3L * e + a] + 1] += 3;
    for (int k = 0; k < nn; k++) deg[k + 1] += deg[k];
    std::vector<int> adj(deg[nn]);
    {
        std::vector<int> fill(deg.begin(), deg.end() - 1);
        for (int e = 0; e < ne; e++)
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) adj[fill[p->tri[3L * e + a]]++] = p->tri[3L * e + b];
    }
    std::vector<int> aptr(nn + 1, 0), acol;
    acol.reserve(deg[nn] / 2 + nn);
    for (int k = 0; k < nn; k++) {
        std::vector<int> v(adj.begin() + deg[k], adj.begin() + deg[k + 1]);
        v.push_back(k);
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        acol.insert(acol.end(), v.begin(), v.end());
        aptr[k + 1] = (int)acol.size();
    }
    // CSR pattern: free row (node k, component q) couples with free dofs of both components of
    // every neighbour; Dirichlet rows hold their diagonal only
    P.ptr.assign(n + 1, 0);
    for (int i = 0; i < n; i++) {
        const int k = i % nn;
        int cnt = 0;
        if (P.fixed[i])
            cnt = 1;
        else
            for (int q = 0; q < nc; q++)
                for (int t = aptr[k]; t < aptr[k + 1]; t++) cnt += P.fixed[q * nn + acol[t]] ? 0 : 1;
        P.ptr[i + 1] = P.ptr[i] + cnt;
    }
    if ((long)P.ptr[n] > (long)INT32_MAX / 4) {
        P.error = "too many entries";
        return false;
    }
    P.col.resize(P.ptr[n]);
    for (int i = 0; i < n; i++) {
        int w = P.ptr[i];
        const int k = i % nn;
        if (P.fixed[i]) {
            P.col[w] = i;
            continue;
        }
        for (int q = 0; q < nc; q++)
            for (int t = aptr[k]; t < aptr[k + 1]; t++) {
                const int j = q * nn + acol[t];
                if (!P.fixed[j]) P.col[w++] = j;
            }
    }
    // contributions, two passes (count, fill), elements in ascending order
    const long nnz = P.ptr[n];
    auto slot = [&](int i, int j) -> long {
        const int* b = P.col.data() + P.ptr[i];
        const int* e = P.col.data() + P.ptr[i + 1];
        const int* f = std::lower_bound(b, e, j);
        return (f != e && *f == j) ? (long)(f - P.col.data()) : -1;
    };
    std::vector<int> ccnt(nnz + 1, 0), lcnt(n + 1, 0);
    for (int i = 0; i < n; i++)
        if (P.fixed[i]) ccnt[P.ptr[i] + 1] = 1;
    auto dof = [&](int e, int a, int c) { return c * nn + p->tri[3L * e + a]; };
    for (int e = 0; e < ne; e++)
        for (int a = 0; a < 3; a++)
            for (int pc = 0; pc < nc; pc++) {
                const int i = dof(e, a, pc);
                if (P.fixed[i]) continue;
                for (int b = 0; b < 3; b++)
                    for (int qc = 0; qc < nc; qc++) {
                        const int j = dof(e, b, qc);
                        if (P.fixed[j])
                            lcnt[i + 1]++;
                        else
                            ccnt[slot(i, j) + 1]++;
                    }
            }
    for (long q = 0; q < nnz; q++) ccnt[q + 1] += ccnt[q];
    for (int i = 0; i < n; i++) lcnt[i + 1] += lcnt[i];
    if ((long)ccnt[nnz] > (long)INT32_MAX) {
        P.error = "too many element contributions";
        return false;
    }
    P.cptr = ccnt;
    P.lptr = lcnt;
    P.celem.resize(ccnt[nnz]);
    P.ccoef.resize(ccnt[nnz]);
    P.lelem.resize(lcnt[n]);
    P.lcoef.resize(lcnt[n]);
    std::vector<int> cf(ccnt.begin(), ccnt.end() - 1), lf(lcnt.begin(), lcnt.end() - 1);
    for (int i = 0; i < n; i++)
        if (P.fixed[i]) {
            const int q = cf[P.ptr[i]]++;
            P.celem[q] = -1;
            P.ccoef[q] = 1.0;
        }
    for (int e = 0; e < ne; e++) {
        Geo g;
        for (int k = 0; k < 3; k++) g.beta[k] = P.geo[7L * e + k], g.gamma[k] = P.geo[7L * e + 3 + k];
        g.area = P.geo[7L * e + 6];
        for (int a = 0; a < 3; a++)
            for (int pc = 0; pc < nc; pc++) {
                const int i = dof(e, a, pc);
                if (P.fixed[i]) continue;
                for (int b = 0; b < 3; b++)
                    for (int qc = 0; qc < nc; qc++) {
                        const int j = dof(e, b, qc);
                        const double k = nc == 2 ? khat(g, P.D, a, pc, b, qc)
                                                 : g.area * (g.beta[a] * g.beta[b] + g.gamma[a] * g.gamma[b]);
                        if (P.fixed[j]) {
                            const int q = lf[i]++;
                            P.lelem[q] = e;
                            P.lcoef[q] = k * P.fixval[j];
                        } else {
                            const int q = cf[slot(i, j)]++;
                            P.celem[q] = e;
                            P.ccoef[q] = k;
                        }
                    }
            }
    }
    return true;
}

// host assembly with the device kernels' arithmetic (each product and sum rounded on its own)
void assemble_host(const Plan& P, const double* E, double* val, double* b) {
    const long nnz = P.ptr[P.n];
    for (long q = 0; q < nnz; q++) {
        double v = 0.0;
        for (int c = P.cptr[q]; c < P.cptr[q + 1]; c++) {
            const double f = P.celem[c] >= 0 ? E[P.celem[c]] : 1.0;
            const double t = f * P.ccoef[c];
            v = v + t;
        }
        val[q] = v;
    }
    for (int i = 0; i < P.n; i++) {
        if (P.fixed[i]) {
            b[i] = P.fixval[i];
            continue;
        }
        double acc = 0.0;
        for (int l = P.lptr[i]; l < P.lptr[i + 1]; l++) {
            const double t = E[P.lelem[l]] * P.lcoef[l];
            acc = acc + t;
        }
        b[i] = -acc;
    }
}

// ---------------------------------------------------------------- kernels
__global__ void assemble_values_kernel(long nnz, const int* __restrict__ cptr, const int* __restrict__ celem,
                                       const double* __restrict__ ccoef, const double* __restrict__ E,
                                       double* __restrict__ val) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (long)gridDim.x * blockDim.x) {
        double v = 0.0;
        const int c1 = cptr[q + 1];
        for (int c = cptr[q]; c < c1; c++) {
            const int e = celem[c];
            v = __dadd_rn(v, __dmul_rn(e >= 0 ? E[e] : 1.0, ccoef[c]));
        }
        val[q] = v;
    }
}

__global__ void assemble_rhs_kernel(int n, const int* __restrict__ lptr, const int* __restrict__ lelem,
                                    const double* __restrict__ lcoef, const unsigned char* __restrict__ fixed,
                                    const double* __restrict__ fixval, const double* __restrict__ E,
                                    double* __restrict__ b) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (fixed[i]) {
            b[i] = fixval[i];
            continue;
        }
        double acc = 0.0;
        for (int l = lptr[i]; l < lptr[i + 1]; l++) acc = __dadd_rn(acc, __dmul_rn(E[lelem[l]], lcoef[l]));
        b[i] = -acc;
    }
}

// L = 1/2 sum_s d_s^2 with d_s = u[dof_s] - target_s, and the adjoint source dL/du (zeroed by the
// caller): one block, fixed summation order
__global__ void loss_kernel(int ns, const int* __restrict__ sdof, const double* __restrict__ target,
                            const double* __restrict__ u, double* __restrict__ src, double* __restrict__ loss) {
    __shared__ double part[kT];
    double acc = 0.0;
    for (int s = threadIdx.x; s < ns; s += blockDim.x) {
        const double d = u[sdof[s]] - target[s];
        src[sdof[s]] = d;
        acc += d * d;
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = 0.5 * part[0];
}

// dL/dE_e = -|T| eps(lambda)^T D eps(u); on Dirichlet dofs lambda is zero and u the known value
__global__ void gradient_kernel(int ne, int nn, const int* __restrict__ tri, const double* __restrict__ geo,
                                const unsigned char* __restrict__ fixed, const double* __restrict__ fixval,
                                const double* __restrict__ u,
                                const double* __restrict__ lam, double d00, double d01, double d11, double d22,
                                double* __restrict__ grad) {
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (long)gridDim.x * blockDim.x) {
        const double* g = geo + 7 * e;
        double eu0 = 0, eu1 = 0, eu2 = 0, el0 = 0, el1 = 0, el2 = 0;
        for (int k = 0; k < 3; k++) {
            const int node = tri[3 * e + k];
            const double b = g[k], c = g[3 + k];
            const double ux = fixed[node] ? fixval[node] : u[node];
            const double uy = fixed[nn + node] ? fixval[nn + node] : u[nn + node];
            const double lx = fixed[node] ? 0.0 : lam[node];
            const double ly = fixed[nn + node] ? 0.0 : lam[nn + node];
            eu0 += b * ux;
            eu1 += c * uy;
            eu2 += c * ux + b * uy;
            el0 += b * lx;
            el1 += c * ly;
            el2 += c * lx + b * ly;
        }
        const double s0 = d00 * eu0 + d01 * eu1;
        const double s1 = d01 * eu0 + d11 * eu1;
        const double s2 = d22 * eu2;
        grad[e] = -g[6] * (el0 * s0 + el1 * s1 + el2 * s2);
    }
}

}  // namespace

// ---------------------------------------------------------------- handle
struct lina_gpu_elastic {
    Plan plan;
    lina_gpu_amg* amg = nullptr;
    cudaStream_t st = nullptr;
    int *d_cptr = nullptr, *d_celem = nullptr, *d_lptr = nullptr, *d_lelem = nullptr, *d_tri = nullptr,
        *d_sdof = nullptr;
    double *d_ccoef = nullptr, *d_lcoef = nullptr, *d_fixval = nullptr, *d_geo = nullptr, *d_target = nullptr;
    unsigned char* d_fixed = nullptr;
    double *d_E = nullptr, *d_val = nullptr, *d_b = nullptr, *d_u = nullptr, *d_lam = nullptr, *d_src = nullptr,
           *d_grad = nullptr, *d_loss = nullptr;
    std::vector<void*> mem;
    int ns = 0;
    bool have_forward = false;
    double last_loss = 0.0;

    ~lina_gpu_elastic() {
        if (amg) lina_gpu_amg_destroy(amg);
        for (void* p : mem) cudaFree(p);
        if (st) cudaStreamDestroy(st);
    }
    template <typename T>
    bool alloc(T** p, size_t count) {
        if (count == 0) count = 1;
        if (cudaMalloc((void**)p, count * sizeof(T)) != cudaSuccess) {
            *p = nullptr;
            return false;
        }
        mem.push_back((void*)*p);
        return true;
    }
    template <typename T>
    bool upload(T** p, const T* src, size_t count) {
        if (!alloc(p, count)) return false;
        return count == 0 || cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, st) == cudaSuccess;
    }
};

namespace {

bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    lina::dev::set_error(buf);
    return false;
}

// assemble A(E) and b on the device from d_E
bool assemble_device(lina_gpu_elastic* h) {
    const Plan& P = h->plan;
    const long nnz = P.ptr[P.n];
    assemble_values_kernel<<<grid(nnz), kT, 0, h->st>>>(nnz, h->d_cptr, h->d_celem, h->d_ccoef, h->d_E, h->d_val);
    assemble_rhs_kernel<<<grid(P.n), kT, 0, h->st>>>(P.n, h->d_lptr, h->d_lelem, h->d_lcoef, h->d_fixed, h->d_fixval,
                                                     h->d_E, h->d_b);
    return cuda_ok(cudaGetLastError(), "assembly launch");
}

}  // namespace

extern "C" {

int lina_gpu_elastic_assemble_host(const lina_gpu_elastic_problem* p, const double* young, int* rowptr, int* col,
                                   double* val, double* b, long* nnz) {
    Plan P;
    if (!check_problem(p, P.error) || !build_plan(mesh_of(p), P)) {
        fail("lina_gpu_elastic_assemble_host: %s", P.error.c_str());
        return LINA_GPU_EINVAL;
    }
    if (nnz) *nnz = P.ptr[P.n];
    if (!rowptr) return 0;
    if (!young || !col || !val || !b) {
        fail("lina_gpu_elastic_assemble_host: missing output");
        return LINA_GPU_EINVAL;
    }
    std::copy(P.ptr.begin(), P.ptr.end(), rowptr);
    std::copy(P.col.begin(), P.col.end(), col);
    assemble_host(P, young, val, b);
    return 0;
}

int lina_gpu_elastic_create(const lina_gpu_elastic_problem* p, const double* young, const lina_gpu_amg_options* opt,
                            lina_gpu_elastic** out) {
    if (!out || !young || !opt) {
        fail("lina_gpu_elastic_create: invalid argument");
        return LINA_GPU_EINVAL;
    }
    *out = nullptr;
    lina_gpu_elastic* h = new lina_gpu_elastic();
    Plan& P = h->plan;
    if (!check_problem(p, P.error) || !build_plan(mesh_of(p), P)) {
        fail("lina_gpu_elastic_create: %s", P.error.c_str());
        delete h;
        return LINA_GPU_EINVAL;
    }
    const long nnz = P.ptr[P.n];
    std::vector<double> val(nnz), b(P.n);
    assemble_host(P, young, val.data(), b.data());
    int rc = lina_gpu_amg_create(P.n, P.ptr.data(), P.col.data(), val.data(), opt, &h->amg);
    if (rc) {
        delete h;
        return rc;
    }
    h->ns = p->n_sensors;
    bool ok = cuda_ok(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking), "stream");
    ok = ok && h->upload(&h->d_cptr, P.cptr.data(), P.cptr.size()) && h->upload(&h->d_celem, P.celem.data(), P.celem.size()) &&
         h->upload(&h->d_ccoef, P.ccoef.data(), P.ccoef.size()) && h->upload(&h->d_lptr, P.lptr.data(), P.lptr.size()) &&
         h->upload(&h->d_lelem, P.lelem.data(), P.lelem.size()) && h->upload(&h->d_lcoef, P.lcoef.data(), P.lcoef.size()) &&
         h->upload(&h->d_fixed, P.fixed.data(), P.fixed.size()) && h->upload(&h->d_fixval, P.fixval.data(), P.fixval.size()) &&
         h->upload(&h->d_geo, P.geo.data(), P.geo.size()) && h->upload(&h->d_tri, p->tri, 3L * P.ne) &&
         h->upload(&h->d_sdof, p->sensor_dof, (size_t)h->ns) && h->upload(&h->d_target, p->target, (size_t)h->ns) &&
         h->upload(&h->d_E, young, (size_t)P.ne) && h->alloc(&h->d_val, nnz) && h->alloc(&h->d_b, P.n) &&
         h->alloc(&h->d_u, P.n) && h->alloc(&h->d_lam, P.n) && h->alloc(&h->d_src, P.n) &&
         h->alloc(&h->d_grad, P.ne) && h->alloc(&h->d_loss, 1);
    ok = ok && cuda_ok(cudaMemsetAsync(h->d_u, 0, P.n * sizeof(double), h->st), "memset") &&
         cuda_ok(cudaStreamSynchronize(h->st), "upload");
    if (!ok) {
        lina::dev::set_error("lina_gpu_elastic_create: device allocation or upload failed");
        delete h;
        return LINA_GPU_ECUDA;
    }
    // the pattern, columns and geometry are kept on the device; the host copies of the
    // contribution lists are no longer needed
    std::vector<int>().swap(P.celem);
    std::vector<double>().swap(P.ccoef);
    std::vector<int>().swap(P.lelem);
    std::vector<double>().swap(P.lcoef);
    std::vector<int>().swap(P.cptr);
    *out = h;
    return 0;
}

int lina_gpu_elastic_forward(lina_gpu_elastic* h, const double* young, double tol, int max_iter, int flags, double* u,
                             double* loss, lina_gpu_solve_info* info) {
    if (!h || !young || max_iter < 1) {
        fail("lina_gpu_elastic_forward: invalid argument");
        return LINA_GPU_EINVAL;
    }
    const Plan& P = h->plan;
    const bool dev = (flags & LINA_PCG_DEVICE_PTRS) != 0;
    if (!cuda_ok(cudaMemcpyAsync(h->d_E, young, P.ne * sizeof(double), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 h->st),
                 "modulus copy"))
        return LINA_GPU_ECUDA;
    if (!assemble_device(h)) return LINA_GPU_ECUDA;
    if (!(flags & LINA_PCG_USE_X0) || !h->have_forward)
        if (!cuda_ok(cudaMemsetAsync(h->d_u, 0, P.n * sizeof(double), h->st), "memset")) return LINA_GPU_ECUDA;
    if (!cuda_ok(cudaStreamSynchronize(h->st), "assembly")) return LINA_GPU_ECUDA;
    int rc;
    if (flags & LINA_ELASTIC_RECOMPUTE) {
        std::vector<double> val(P.ptr[P.n]);
        if (!cuda_ok(cudaMemcpy(val.data(), h->d_val, val.size() * sizeof(double), cudaMemcpyDeviceToHost), "copy"))
            return LINA_GPU_ECUDA;
        rc = lina_gpu_amg_recompute(h->amg, P.n, P.ptr.data(), P.col.data(), val.data());
    } else {
        rc = lina_gpu_amg_update_values(h->amg, h->d_val, LINA_PCG_DEVICE_PTRS);
    }
    if (rc) return rc;
    lina_gpu_solve_info local;
    lina_gpu_solve_info* in = info ? info : &local;
    rc = lina_gpu_pcg(h->amg, h->d_b, h->d_u, tol, max_iter, LINA_STOP_RELATIVE,
                      LINA_PCG_DEVICE_PTRS | LINA_PCG_USE_X0, in);
    h->have_forward = true;
    if (rc < 0 && rc != LINA_GPU_ENOCONV) return rc;
    if (!cuda_ok(cudaMemsetAsync(h->d_src, 0, P.n * sizeof(double), h->st), "memset")) return LINA_GPU_ECUDA;
    loss_kernel<<<1, kT, 0, h->st>>>(h->ns, h->d_sdof, h->d_target, h->d_u, h->d_src, h->d_loss);
    if (!cuda_ok(cudaGetLastError(), "loss launch")) return LINA_GPU_ECUDA;
    if (!cuda_ok(cudaMemcpyAsync(&h->last_loss, h->d_loss, sizeof(double), cudaMemcpyDeviceToHost, h->st), "copy"))
        return LINA_GPU_ECUDA;
    if (u && !cuda_ok(cudaMemcpyAsync(u, h->d_u, P.n * sizeof(double), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                      h->st),
                      "copy"))
        return LINA_GPU_ECUDA;
    if (!cuda_ok(cudaStreamSynchronize(h->st), "forward")) return LINA_GPU_ECUDA;
    if (loss) *loss = h->last_loss;
    return rc;
}

int lina_gpu_elastic_backward(lina_gpu_elastic* h, double tol, int max_iter, int flags, double* grad, double* lambda,
                              lina_gpu_solve_info* info) {
    if (!h || !grad || max_iter < 1 || !h->have_forward) {
        fail("lina_gpu_elastic_backward: invalid argument (or no forward pass yet)");
        return LINA_GPU_EINVAL;
    }
    const Plan& P = h->plan;
    const bool dev = (flags & LINA_PCG_DEVICE_PTRS) != 0;
    int rc = 0;
    lina_gpu_solve_info local;
    lina_gpu_solve_info* in = info ? info : &local;
    if (h->last_loss == 0.0) {  // dL/du = 0: lambda = 0, no solve
        memset(in, 0, sizeof *in);
        if (!cuda_ok(cudaMemsetAsync(h->d_lam, 0, P.n * sizeof(double), h->st), "memset")) return LINA_GPU_ECUDA;
    } else {
        rc = lina_gpu_pcg(h->amg, h->d_src, h->d_lam, tol, max_iter, LINA_STOP_RELATIVE, LINA_PCG_DEVICE_PTRS, in);
        if (rc < 0 && rc != LINA_GPU_ENOCONV) return rc;
    }
    gradient_kernel<<<grid(P.ne), kT, 0, h->st>>>(P.ne, P.nn, h->d_tri, h->d_geo, h->d_fixed, h->d_fixval, h->d_u, h->d_lam, P.D.d00,
                                                  P.D.d01, P.D.d11, P.D.d22, h->d_grad);
    if (!cuda_ok(cudaGetLastError(), "gradient launch")) return LINA_GPU_ECUDA;
    const cudaMemcpyKind k = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (!cuda_ok(cudaMemcpyAsync(grad, h->d_grad, P.ne * sizeof(double), k, h->st), "copy")) return LINA_GPU_ECUDA;
    if (lambda && !cuda_ok(cudaMemcpyAsync(lambda, h->d_lam, P.n * sizeof(double), k, h->st), "copy"))
        return LINA_GPU_ECUDA;
    if (!cuda_ok(cudaStreamSynchronize(h->st), "backward")) return LINA_GPU_ECUDA;
    return rc;
}

int lina_gpu_elastic_sizes(const lina_gpu_elastic* h, int* n, long* nnz) {
    if (!h) return LINA_GPU_EINVAL;
    if (n) *n = h->plan.n;
    if (nnz) *nnz = h->plan.ptr[h->plan.n];
    return 0;
}

int lina_gpu_elastic_system(lina_gpu_elastic* h, int* rowptr, int* col, double* val, double* b) {
    if (!h) return LINA_GPU_EINVAL;
    const Plan& P = h->plan;
    if (rowptr) std::copy(P.ptr.begin(), P.ptr.end(), rowptr);
    if (col) std::copy(P.col.begin(), P.col.end(), col);
    if (!h->have_forward && (val || b)) {  // the creation matrix: assemble it from the stored moduli
        if (!assemble_device(h)) return LINA_GPU_ECUDA;
    }
    if (val && !cuda_ok(cudaMemcpyAsync(val, h->d_val, P.ptr[P.n] * sizeof(double), cudaMemcpyDeviceToHost, h->st), "copy"))
        return LINA_GPU_ECUDA;
    if (b && !cuda_ok(cudaMemcpyAsync(b, h->d_b, P.n * sizeof(double), cudaMemcpyDeviceToHost, h->st), "copy"))
        return LINA_GPU_ECUDA;
    return cuda_ok(cudaStreamSynchronize(h->st), "system copy") ? 0 : LINA_GPU_ECUDA;
}

lina_gpu_amg* lina_gpu_elastic_amg(lina_gpu_elastic* h) { return h ? h->amg : nullptr; }

int lina_gpu_elastic_destroy(lina_gpu_elastic* h) {
    delete h;
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- general P1 assembly
struct lina_gpu_p1 {
    Plan plan;
    cudaStream_t st = nullptr;
    int *d_cptr = nullptr, *d_celem = nullptr, *d_lptr = nullptr, *d_lelem = nullptr;
    double *d_ccoef = nullptr, *d_lcoef = nullptr, *d_fixval = nullptr, *d_coef = nullptr, *d_val = nullptr,
           *d_b = nullptr;
    unsigned char* d_fixed = nullptr;
    std::vector<void*> mem;
    bool assembled = false;

    ~lina_gpu_p1() {
        if (st) cudaStreamSynchronize(st);
        for (void* p : mem) cudaFree(p);
        if (st) cudaStreamDestroy(st);
    }
    template <typename T>
    bool alloc(T** p, size_t count) {
        if (count == 0) count = 1;
        if (cudaMalloc((void**)p, count * sizeof(T)) != cudaSuccess) {
            *p = nullptr;
            return false;
        }
        mem.push_back((void*)*p);
        return true;
    }
    template <typename T>
    bool upload(T** p, const T* src, size_t count) {
        if (!alloc(p, count)) return false;
        return count == 0 || cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, st) == cudaSuccess;
    }
};

namespace {

Mesh mesh_of(const lina_gpu_p1_problem* p) {
    Mesh m;
    if (!p) {
        m.kind = 0;
        return m;
    }
    m.kind = p->kind;
    m.nn = p->n_nodes;
    m.ne = p->n_elems;
    m.xy = p->xy;
    m.tri = p->tri;
    m.nu = p->nu;
    m.n_fixed = p->n_fixed;
    m.fixed_dof = p->fixed_dof;
    m.fixed_val = p->fixed_val;
    return m;
}

}  // namespace

extern "C" {

int lina_gpu_p1_create(const lina_gpu_p1_problem* p, lina_gpu_p1** out) {
    if (!out) return LINA_GPU_EINVAL;
    *out = nullptr;
    lina_gpu_p1* h = new lina_gpu_p1();
    Plan& P = h->plan;
    if (!build_plan(mesh_of(p), P)) {
        fail("lina_gpu_p1_create: %s", P.error.c_str());
        delete h;
        return LINA_GPU_EINVAL;
    }
    const long nnz = P.ptr[P.n];
    bool ok = cuda_ok(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking), "stream");
    ok = ok && h->upload(&h->d_cptr, P.cptr.data(), P.cptr.size()) &&
         h->upload(&h->d_celem, P.celem.data(), P.celem.size()) &&
         h->upload(&h->d_ccoef, P.ccoef.data(), P.ccoef.size()) && h->upload(&h->d_lptr, P.lptr.data(), P.lptr.size()) &&
         h->upload(&h->d_lelem, P.lelem.data(), P.lelem.size()) &&
         h->upload(&h->d_lcoef, P.lcoef.data(), P.lcoef.size()) &&
         h->upload(&h->d_fixed, P.fixed.data(), P.fixed.size()) &&
         h->upload(&h->d_fixval, P.fixval.data(), P.fixval.size()) && h->alloc(&h->d_coef, (size_t)P.ne) &&
         h->alloc(&h->d_val, (size_t)nnz) && h->alloc(&h->d_b, (size_t)P.n) &&
         cuda_ok(cudaStreamSynchronize(h->st), "upload");
    if (!ok) {
        fail("lina_gpu_p1_create: device allocation or upload failed");
        delete h;
        return LINA_GPU_ECUDA;
    }
    *out = h;
    return 0;
}

int lina_gpu_p1_assemble(lina_gpu_p1* h, const double* coef, int flags) {
    if (!h || !coef) return LINA_GPU_EINVAL;
    const Plan& P = h->plan;
    const double* c = coef;
    if (!(flags & LINA_PCG_DEVICE_PTRS)) {
        if (!cuda_ok(cudaMemcpyAsync(h->d_coef, coef, P.ne * sizeof(double), cudaMemcpyHostToDevice, h->st), "copy"))
            return LINA_GPU_ECUDA;
        c = h->d_coef;
    }
    const long nnz = P.ptr[P.n];
    assemble_values_kernel<<<grid(nnz), kT, 0, h->st>>>(nnz, h->d_cptr, h->d_celem, h->d_ccoef, c, h->d_val);
    assemble_rhs_kernel<<<grid(P.n), kT, 0, h->st>>>(P.n, h->d_lptr, h->d_lelem, h->d_lcoef, h->d_fixed, h->d_fixval, c,
                                                     h->d_b);
    if (!cuda_ok(cudaGetLastError(), "assembly") || !cuda_ok(cudaStreamSynchronize(h->st), "assembly"))
        return LINA_GPU_ECUDA;
    h->assembled = true;
    return 0;
}

int lina_gpu_p1_sizes(const lina_gpu_p1* h, int* n, long* nnz) {
    if (!h) return LINA_GPU_EINVAL;
    if (n) *n = h->plan.n;
    if (nnz) *nnz = h->plan.ptr[h->plan.n];
    return 0;
}

int lina_gpu_p1_download(lina_gpu_p1* h, int* rowptr, int* col, double* val, double* b) {
    if (!h) return LINA_GPU_EINVAL;
    const Plan& P = h->plan;
    if (rowptr) std::copy(P.ptr.begin(), P.ptr.end(), rowptr);
    if (col) std::copy(P.col.begin(), P.col.end(), col);
    if ((val || b) && !h->assembled) {
        fail("lina_gpu_p1_download: nothing assembled yet");
        return LINA_GPU_EINVAL;
    }
    if (val && !cuda_ok(cudaMemcpyAsync(val, h->d_val, P.ptr[P.n] * sizeof(double), cudaMemcpyDeviceToHost, h->st), "copy"))
        return LINA_GPU_ECUDA;
    if (b && !cuda_ok(cudaMemcpyAsync(b, h->d_b, P.n * sizeof(double), cudaMemcpyDeviceToHost, h->st), "copy"))
        return LINA_GPU_ECUDA;
    return cuda_ok(cudaStreamSynchronize(h->st), "copy") ? 0 : LINA_GPU_ECUDA;
}

int lina_gpu_p1_device(lina_gpu_p1* h, const double** val_dev, const double** b_dev) {
    if (!h || !h->assembled) return LINA_GPU_EINVAL;
    if (val_dev) *val_dev = h->d_val;
    if (b_dev) *b_dev = h->d_b;
    return 0;
}

int lina_gpu_p1_destroy(lina_gpu_p1* h) {
    delete h;
    return 0;
}

int lina_gpu_p1_assemble_host(const lina_gpu_p1_problem* p, const double* coef, int* rowptr, int* col, double* val,
                              double* b, long* nnz) {
    Plan P;
    if (!build_plan(mesh_of(p), P)) {
        fail("lina_gpu_p1_assemble_host: %s", P.error.c_str());
        return LINA_GPU_EINVAL;
    }
    if (nnz) *nnz = P.ptr[P.n];
    if (!rowptr) return 0;
    if (!coef || !col || !val || !b) {
        fail("lina_gpu_p1_assemble_host: missing output");
        return LINA_GPU_EINVAL;
    }
    std::copy(P.ptr.begin(), P.ptr.end(), rowptr);
    std::copy(P.col.begin(), P.col.end(), col);
    assemble_host(P, coef, val, b);
    return 0;
}

}  // extern "C"
