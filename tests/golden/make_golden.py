"""Generate the committed golden fixtures from the reference LinA itself.

Run in a checkout where the reference tree is available (``make -C oracle ref``
builds oracle/_ref/libLinA_ref.so from it):

    python tests/golden/make_golden.py [case ...]

For each small seeded system it records what the reference computes:
the AMG hierarchy of AMG_setup (LinA/Multigrid.c:1613) level by level (C/F
labels, A, P, R), the greedy colouring of each level, one preconditioner
application (a V-cycle from the zero guess) for a seeded residual, and full
pcg solves (LinA/PCGS.c:163) with the smoothers the GPU library implements
(installed into the reference through AMG_set_smoother) and with the
reference's own lexicographic SOR.  For bound-constrained damage quadratics
it records the minimiser and iteration count of reflective_newton with two
of the reference's local solvers; and for a material-identification case the
forward solutions and the adjoint solved with the reference's transpose of A.  The P1 assembly
fixture records FEM2D's own stiffness matrices (``make -C oracle fem2d``) on stored meshes.
Tests compare the GPU library against
these files on machines where the reference is absent.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fem_gb300 import problems  # noqa: E402
from oracle import ref  # noqa: E402

# name -> (system factory, depth, coarsening)
CASES = {
    "poisson33_aggr": (lambda: problems.poisson_p1(33, seed=0), 4, ref.AGGRESSIVE),
    "poisson33_std": (lambda: problems.poisson_p1(33, seed=0), 4, ref.STANDARD),
    "elast17_aggr": (lambda: problems.elasticity_p1(17), 3, ref.AGGRESSIVE),
    "elast17_std": (lambda: problems.elasticity_p1(17), 3, ref.STANDARD),
    # two levels: a coarsest dense block of about 2,000 rows (the GPU inverts it at set-up)
    "poisson65_d2": (lambda: problems.poisson_p1(65, seed=0), 2, ref.STANDARD),
}
# larger systems for which only the solves are stored (the input is regenerated
# by fem_gb300.problems and checked against the stored digest)
SOLVE_CASES = {
    "poisson129_aggr_solve": (lambda: problems.poisson_p1(129, seed=0), 5, ref.AGGRESSIVE),
    "elast65_std_solve": (lambda: problems.elasticity_p1(65), 5, ref.STANDARD),
}
# smoother configurations: name -> (reference smoother kind, omega)
SMOOTHERS = {
    "jacobi": (ref.SMOOTHER_DAMPED_JACOBI, 0.6),
    "mcsor": (ref.SMOOTHER_MC_SOR, 1.0),
    "refsor": (ref.SMOOTHER_REF_SOR, 1.0),
}
TOL = 1e-8
MAX_IT = 500
# configuration-size systems, stored as digests (per-level SHA-256 of the hierarchy, iteration
# counts, norms and a fixed subsample of each solution; tests/golden/digest.py): the 2.1M-unknown
# degraded elasticity system of the benchmark (standard coarsening, depth 10) and the 66,049-unknown
# Poisson system (aggressive coarsening, depth 6, lexicographic SOR with omega 1)
DIGEST_CASES = {
    "elast1025_digest": (lambda: problems.elasticity_p1(1025), 10, ref.STANDARD, ("jacobi", "refsor")),
    "poisson257_digest": (lambda: problems.poisson_p1(257, seed=0), 6, ref.AGGRESSIVE, ("refsor", "jacobi", "mcsor")),
}
# the AT2 damage step at 1025 x 1025 nodes (1.05M unknowns) by reflective Newton, stored as a digest
RN_DIGEST_CASES = {"at2_1025_rn_digest": lambda: problems.at2_damage(1025)}
# bound-constrained damage quadratics solved by reflective_newton (LinA/reflective_newton.c:660)
RN_CASES = {
    "damage65_rn": lambda: problems.damage_qp(65),
    "damage129_rn": lambda: problems.damage_qp(129),
    "at2_65_rn": lambda: problems.at2_damage(65),
}
# bound-constrained quadratics with an indefinite Hessian: the local solve reports INDEFINITE and
# reflective_newton takes the direction of negative curvature; solved with the complete Cholesky local
# solver (RN_CHOLESKY) and with BiCGStab + ILU(0) in the RN_UMF slot
INDEF_CASES = {"indef17_rn": lambda: problems.indefinite_qp(17)}
INDEF_SOLVERS = {"cholesky": 4, "umf_bicgstab_ilu": 5}
# material identification (adjoint) cases: name -> (grid size m, AMG depth)
ADJOINT_CASES = {"adjoint65": (65, 5)}
# gmres / Newton_solver / active_set_solver runs of the reference, one file
SOLVERS_FILE = "solvers"
# reference local solvers: name -> RN solver code (5 = RN_UMF slot running BiCGStab + ILU(0), 3 = RN_PCG)
RN_SOLVERS = {"umf_bicgstab_ilu": 5, "pcg_ilu": 3}


def system_digest(s) -> str:
    h = hashlib.sha256()
    for a in (s.indptr, s.indices, s.data, s.b):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make_case(name):
    factory, depth, coarsening = CASES[name]
    s = factory()
    amg = ref.RefAMG(s, depth, 2, 2, coarsening)
    out = {
        "n": np.int64(s.n), "dof": np.int64(s.dof), "depth": np.int64(depth),
        "coarsening": np.int64(coarsening), "digest": np.array(system_digest(s)),
        "indptr": s.indptr, "indices": s.indices, "data": s.data, "b": s.b,
        "sizes": np.array(amg.sizes(), dtype=np.int64),
    }
    for lv in range(depth):
        L = amg.level(lv)
        out[f"L{lv}_A_ptr"], out[f"L{lv}_A_col"], out[f"L{lv}_A_val"] = L.A
        if lv > 0:
            out[f"L{lv}_labels"] = L.labels
            out[f"L{lv}_P_ptr"], out[f"L{lv}_P_col"], out[f"L{lv}_P_val"] = L.P
            out[f"L{lv}_R_ptr"], out[f"L{lv}_R_col"], out[f"L{lv}_R_val"] = L.R
            nc, col = ref.greedy_colouring(len(L.A[0]) - 1, *L.A)
            out[f"L{lv}_colour"] = col
    rng = np.random.default_rng(1)
    r = rng.uniform(-1.0, 1.0, s.n)
    out["vcycle_r"] = r
    for sname, (kind, omega) in SMOOTHERS.items():
        out[f"vcycle_{sname}"] = amg.vcycle(r, kind, omega)
        x, it, res = amg.pcg(s.b, TOL, MAX_IT, kind, omega)
        out[f"pcg_{sname}_x"] = x
        out[f"pcg_{sname}_it"] = np.int64(it)
        out[f"pcg_{sname}_res"] = np.float64(res)
    # an accurate FP64 solution (reference pcg to a tight tolerance) for error bars
    x, it, res = amg.pcg(s.b, 1e-13, 2000, ref.SMOOTHER_MC_SOR, 1.0)
    out["x_tight"] = x
    # AMG_solve alone (V-cycles to 1e-8) with damped Jacobi
    x, it = amg.amg_solve(s.b, 1e-8, 200, ref.SMOOTHER_DAMPED_JACOBI, 0.6)
    out["amgsolve_jacobi_x"] = x
    out["amgsolve_jacobi_it"] = np.int64(it)
    # the reference's stock AMG preconditioner (PCG_set_AMG_preconditioner: aggressive coarsening,
    # 2+3 sweeps, up to 100 warm-started V-cycles to 1e-2) with multicolour SOR, omega 1.6
    x, it, res = ref.pcg_stock(s, depth, ref.SMOOTHER_MC_SOR, 1.6)
    out["stock_x"] = x
    out["stock_it"] = np.int64(it)
    out["stock_res"] = np.float64(res)
    # ILU(0) preconditioner application and BiCGStab with it
    out["ilu_z"] = ref.ilu_apply(s, r)
    x, it = ref.bicgstab_ilu(s, 1e-8, 1000)
    out["bicgstab_ilu_x"] = x
    out["bicgstab_ilu_it"] = np.int64(it)
    return out


def make_solve_case(name):
    factory, depth, coarsening = SOLVE_CASES[name]
    s = factory()
    amg = ref.RefAMG(s, depth, 2, 2, coarsening)
    out = {"n": np.int64(s.n), "dof": np.int64(s.dof), "depth": np.int64(depth),
           "coarsening": np.int64(coarsening), "digest": np.array(system_digest(s)),
           "indptr": s.indptr, "indices": s.indices, "data": s.data, "b": s.b,
           "sizes": np.array(amg.sizes(), dtype=np.int64)}
    for sname, (kind, omega) in SMOOTHERS.items():
        if sname == "refsor":
            continue
        x, it, res = amg.pcg(s.b, TOL, MAX_IT, kind, omega)
        out[f"pcg_{sname}_x"] = x
        out[f"pcg_{sname}_it"] = np.int64(it)
        out[f"pcg_{sname}_res"] = np.float64(res)
    x, it, res = amg.pcg(s.b, 1e-13, 2000, ref.SMOOTHER_MC_SOR, 1.0)
    out["x_tight"] = x
    return out


def make_digest_case(name):
    import time
    from tests.golden import digest as D
    factory, depth, coarsening, smoothers = DIGEST_CASES[name]
    s = factory()
    t0 = time.perf_counter()
    amg = ref.RefAMG(s, depth, 2, 2, coarsening)
    t_setup = time.perf_counter() - t0
    idx = D.sample_index(s.n)
    out = {"n": np.int64(s.n), "dof": np.int64(s.dof), "depth": np.int64(depth),
           "coarsening": np.int64(coarsening), "digest": np.array(system_digest(s)),
           "sizes": np.array(amg.sizes(), dtype=np.int64), "sample_index": idx,
           "ref_setup_s": np.float64(t_setup)}
    for k, v in D.level_digest(amg.level, depth).items():
        out[f"sha_{k}"] = np.array(v)
    bn = np.linalg.norm(s.b)
    import scipy.sparse as sp
    A = sp.csr_matrix((s.data, s.indices, s.indptr), shape=(s.n, s.n))
    for sname in smoothers:
        kind, omega = SMOOTHERS[sname]
        t0 = time.perf_counter()
        x, it, res = amg.pcg(s.b, TOL, MAX_IT, kind, omega)
        out[f"pcg_{sname}_s"] = np.float64(time.perf_counter() - t0)
        out[f"pcg_{sname}_it"] = np.int64(it)
        out[f"pcg_{sname}_res"] = np.float64(res)
        out[f"pcg_{sname}_norm"] = np.float64(np.linalg.norm(x))
        out[f"pcg_{sname}_true_rel"] = np.float64(np.linalg.norm(s.b - A @ x) / bn)
        out[f"pcg_{sname}_xs"] = x[idx]
        print(f"  {name} {sname}: {it} iterations, {out[f'pcg_{sname}_s']:.1f} s", flush=True)
    # an accurate FP64 solution (tolerance 1e-13 in the reference's rule) for error bars
    kind, omega = SMOOTHERS[smoothers[0]]
    x, it, res = amg.pcg(s.b, 1e-13, 4000, kind, omega)
    out["tight_it"] = np.int64(it)
    out["tight_norm"] = np.float64(np.linalg.norm(x))
    out["tight_xs"] = x[idx]
    if s.n <= 100_000:
        out["x_tight"] = x
    return out


def make_rn_digest_case(name):
    import time
    from tests.golden import digest as D
    q = RN_DIGEST_CASES[name]()
    idx = D.sample_index(q.n)
    out = {"n": np.int64(q.n), "sample_index": idx,
           "digest": np.array(system_digest(q))}
    for sname, code in RN_SOLVERS.items():
        if code != 5:
            continue
        t0 = time.perf_counter()
        x, it = ref.reflective_newton_qp(q, solver=code, max_iter=50, eps=1e-8, bi_eps=1e-8)
        out[f"rn_{sname}_s"] = np.float64(time.perf_counter() - t0)
        out[f"rn_{sname}_it"] = np.int64(it)
        out[f"rn_{sname}_norm"] = np.float64(np.linalg.norm(x))
        out[f"rn_{sname}_xs"] = x[idx]
        out[f"rn_{sname}_min"] = np.float64(x.min())
        out[f"rn_{sname}_max"] = np.float64(x.max())
        lo, up = q.meta["lower"], q.meta["upper"]
        out[f"rn_{sname}_at_lower"] = np.int64(np.sum(np.abs(x - lo) <= 1e-10))
        out[f"rn_{sname}_at_upper"] = np.int64(np.sum(np.abs(x - up) <= 1e-10))
    return out


def make_indef_case(name):
    q = INDEF_CASES[name]()
    out = {"n": np.int64(q.n), "indptr": q.indptr, "indices": q.indices, "data": q.data, "b": q.b,
           "lower": q.meta["lower"], "upper": q.meta["upper"], "x0": q.meta["x0"]}
    for sname, code in INDEF_SOLVERS.items():
        x, it = ref.reflective_newton_qp(q, solver=code, max_iter=50, eps=1e-8, bi_eps=1e-8)
        out[f"rn_{sname}_x"] = x
        out[f"rn_{sname}_it"] = np.int64(it)
        out[f"rn_{sname}_negcurv"] = np.int64(ref.rn_neg_curv())
    return out


def make_rn_case(name):
    q = RN_CASES[name]()
    out = {"n": np.int64(q.n), "indptr": q.indptr, "indices": q.indices, "data": q.data, "b": q.b,
           "lower": q.meta["lower"], "upper": q.meta["upper"], "x0": q.meta["x0"]}
    for sname, code in RN_SOLVERS.items():
        x, it = ref.reflective_newton_qp(q, solver=code, max_iter=50, eps=1e-8, bi_eps=1e-8)
        out[f"rn_{sname}_x"] = x
        out[f"rn_{sname}_it"] = np.int64(it)
    return out


def _ref_solve(s, depth, rhs):
    amg = ref.RefAMG(s, depth, 2, 2, ref.STANDARD)
    x, it, _ = amg.pcg(rhs, 1e-13, 2000, ref.SMOOTHER_MC_SOR, 1.0)
    return x, it


def make_adjoint_case(name):
    """Forward solves for the target and actual moduli, then the adjoint solve on the reference's
    own transpose of A (get_transpose, LinA/linear_algebra.c:1290), all with the reference's pcg."""
    m, depth = ADJOINT_CASES[name]
    case = problems.adjoint_case(m, seed=0)
    _, _, fixed_dof, fixed_val = problems.elastic_mesh(m)
    sd = case["sensor_dof"]
    st = problems.elasticity_p1(m, young=case["young_target"].reshape(2, -1))
    ut, it_t = _ref_solve(st, depth, st.b)
    target = ut[sd]
    s = problems.elasticity_p1(m, young=case["young"].reshape(2, -1))
    u, it_u = _ref_solve(s, depth, s.b)
    u[fixed_dof] = fixed_val
    src = np.zeros(s.n)
    src[sd] = u[sd] - target
    loss = 0.5 * float(np.sum(src[sd] ** 2))
    At = ref.RefMatrix.from_csr(s.n, s.indptr, s.indices, s.data).transpose()
    ip_, ix_, dv_ = At.to_csr()
    sT = problems.CSRSystem(s.n, ip_, ix_, dv_, src, dof=2)
    lam, it_l = _ref_solve(sT, depth, src)
    lam[fixed_dof] = 0.0
    grad = problems.element_gradient(m, u, lam)
    return {"m": np.int64(m), "depth": np.int64(depth), "young": case["young"], "young_target": case["young_target"],
            "sensor_dof": sd, "target": target, "u": u, "lam": lam, "grad": grad, "loss": np.float64(loss),
            "it": np.array([it_t, it_u, it_l], dtype=np.int64)}


def spgemm_inputs(seed=7):
    """Seeded rectangular CSR factors with explicit zeros, empty rows and exactly cancelling
    products, as (indptr, indices, data) triples: A is 300 x 200, B is 200 x 150."""
    rng = np.random.default_rng(seed)

    def rand_csr(n, m, density, zero_rows):
        rows = []
        for i in range(n):
            if i in zero_rows:
                rows.append(([], []))
                continue
            k = rng.binomial(m, density)
            cols = np.sort(rng.choice(m, size=k, replace=False))
            vals = rng.standard_normal(k)
            vals[rng.random(k) < 0.1] = 0.0  # explicit zeros
            rows.append((cols, vals))
        return rows

    A = rand_csr(300, 200, 0.04, {5, 17, 123})
    B = rand_csr(200, 150, 0.05, {3, 44})
    # rows 10 and 11 of B are equal; row 7 of A takes +1 x row 10 and -1 x row 11: exact cancellation
    B[11] = (np.array(B[10][0]), np.array(B[10][1]))
    A[7] = (np.array([10, 11]), np.array([1.0, -1.0]))

    def pack(rows):
        ptr = np.zeros(len(rows) + 1, np.int32)
        for i, (c, _) in enumerate(rows):
            ptr[i + 1] = ptr[i] + len(c)
        col = np.concatenate([np.asarray(c, np.int32) for c, _ in rows]).astype(np.int32)
        val = np.concatenate([np.asarray(v, np.float64) for _, v in rows])
        return ptr, col, val

    return pack(A), pack(B)


ILU_FILE = "ilu"
BATCH_FILE = "batch_small"
# small systems of the batched workload: name -> (kind, dofs, seed)
BATCH_CASES = {"bpoisson3k": ("poisson", 3000, 11), "belast4k": ("elasticity", 4000, 12),
               "bpoisson12k": ("poisson", 12000, 13)}


def make_batch():
    """pcg of the reference (damped-Jacobi V-cycle, tolerance 1e-8 in its own rule) and an accurate
    solution (1e-13) for small systems of the batched unstructured workload; the systems are stored."""
    out = {}
    for name, (kind, dofs, seed) in BATCH_CASES.items():
        s = problems.batch_system(kind, dofs, seed)
        depth = problems.batch_depth(s.n)
        amg = ref.RefAMG(s, depth, 2, 2, ref.STANDARD)
        x, it, res = amg.pcg(s.b, TOL, MAX_IT, ref.SMOOTHER_DAMPED_JACOBI, 0.6)
        xt, _, _ = amg.pcg(s.b, 1e-13, 2000, ref.SMOOTHER_MC_SOR, 1.0)
        out.update({f"{name}_ptr": s.indptr, f"{name}_col": s.indices, f"{name}_val": s.data, f"{name}_b": s.b,
                    f"{name}_dof": np.int64(s.dof), f"{name}_depth": np.int64(depth), f"{name}_x": x,
                    f"{name}_it": np.int64(it), f"{name}_x_tight": xt})
    return out


def ilu_inputs():
    """Matrices for the ILU(0) factors: name -> (indptr, indices, data).  Besides the model
    problems, a seeded nonsymmetric matrix with ragged rows (rows holding only the diagonal, rows
    with up to 12 entries) and a 3 x 3 matrix whose second pivot is exactly zero."""
    out = {}
    for name, s in (("poisson33", problems.poisson_p1(33, seed=0)), ("elast17", problems.elasticity_p1(17)),
                    ("damage65", problems.damage_qp(65))):
        out[name] = (s.indptr, s.indices, s.data)
    rng = np.random.default_rng(21)
    n = 400
    rows = []
    for i in range(n):
        k = int(rng.integers(0, 12)) if i % 7 else 0
        cols = set(int(c) for c in rng.integers(max(0, i - 40), min(n, i + 40), size=k)) | {i}
        rows.append(sorted(cols))
    ptr = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    col = np.array([c for r in rows for c in r], dtype=np.int32)
    val = rng.standard_normal(len(col))
    for i in range(n):
        d = ptr[i] + rows[i].index(i)
        val[d] = 4.0 + 4.0 * rng.random()
    out["nonsym400"] = (ptr, col, val)
    out["zeropivot3"] = (np.array([0, 2, 5, 7], dtype=np.int32), np.array([0, 1, 0, 1, 2, 1, 2], dtype=np.int32),
                         np.array([1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0]))
    return out


def make_ilu():
    """incomplete_LU_factorization (LinA/linear_algebra.c:1952) of the reference on ilu_inputs()."""
    out = {}
    for name, (ptr, col, val) in ilu_inputs().items():
        n = len(ptr) - 1
        ok, f = ref.ilu_factors(n, ptr, col, val)
        out[f"{name}_ptr"], out[f"{name}_col"], out[f"{name}_val"] = ptr, col, val
        out[f"{name}_ok"] = np.int64(ok)
        if ok:
            out[f"{name}_f"] = f
    return out


def make_spgemm():
    """sparse_product (LinA/linear_algebra.c:186) of the reference on spgemm_inputs()."""
    (ap, ac, av), (bp, bc, bv) = spgemm_inputs()
    A = ref.RefMatrix.from_csr(len(ap) - 1, ap, ac, av)
    B = ref.RefMatrix.from_csr(len(bp) - 1, bp, bc, bv)
    C = ref.RefMatrix(ref.lib().rs_product(A.ptr, B.ptr))
    cp, cc, cv = C.to_csr()
    return {"a_ptr": ap, "a_col": ac, "a_val": av, "b_ptr": bp, "b_col": bc, "b_val": bv,
            "c_ptr": cp, "c_col": cc, "c_val": cv}


def make_fmg():
    """One full-multigrid pass (AMG_solve with FULL_AMG) of the reference for every hierarchy case
    and the GPU smoothers."""
    out = {}
    for name, (factory, depth, coarsening) in CASES.items():
        s = factory()
        amg = ref.RefAMG(s, depth, 2, 2, coarsening)
        for sname, (kind, omega) in SMOOTHERS.items():
            if sname == "refsor":
                continue
            out[f"{name}_{sname}"] = amg.fmg(s.b, smoother=kind, omega=omega)
    return out


def make_solvers():
    """gmres with ILU(0) right preconditioning (both termination checks), Newton_solver on a cubic
    reaction-diffusion problem (ILU-GMRES and sparse-LU steps) and active_set_solver on a
    box-constrained Poisson problem, all run by the reference."""
    out = {}
    systems = {"poisson33": problems.poisson_p1(33, seed=0), "elast17": problems.elasticity_p1(17)}
    for name, s in systems.items():
        for check in (0, 1):
            tol = 1e-8 if name == "poisson33" else 1e-10
            y, it, rc, nmv, prec = ref.gmres(s, tol=tol, i_max=20, maxiter=1000, check_each=bool(check))
            key = f"gmres_{name}_{check}"
            out[key + "_y"], out[key + "_it"], out[key + "_rc"] = y, np.int64(it), np.int64(rc)
            out[key + "_nomatvec"], out[key + "_precision"] = np.int64(nmv), np.float64(prec)
            out[key + "_tol"] = np.float64(tol)
            out[key + "_x"] = ref.ilu_apply(s, y)  # x = B_r y with the reference's ILU(0)
    s = problems.poisson_p1(17, seed=2)
    B = 10.0 * s.b
    for mode in (0, 1):
        X, it = ref.newton(s, 50.0, B, np.zeros(s.n), maxiter=50, eps=1e-10, mode=mode, i_max=20)
        out[f"newton_{mode}_x"], out[f"newton_{mode}_it"] = X, np.int64(it)
    out["newton_B"] = B
    s = problems.poisson_p1(17, seed=1)
    lo, up = np.full(s.n, -0.002), np.full(s.n, 0.002)
    x, it, na = ref.active_set(s, lo, up, max_iter=100)
    out["active_x"], out["active_it"], out["active_size"] = x, np.int64(it), np.int64(na)
    out["active_lower"], out["active_upper"] = lo, up
    return out


P1_FILE = "p1_fem2d"
# meshes of the P1 assembly fixture: structured grids of the elasticity benchmark and seeded Delaunay
# meshes of the batched workload (stored with the file: scipy's triangulation may differ between hosts)
P1_MESHES = {"grid17": lambda: problems.elastic_mesh(17)[:2], "delaunay600": lambda: problems.delaunay_mesh(600, 5)}


def make_p1():
    """The reference's own P1 assembly (FEM2D set_matrix_Aij_11_2D, oracle/fem2d_shim.c): the Laplacian
    with coefficient 1 and plane-strain elasticity (E 210, nu 0.3, assembled as crack.c does) on each
    mesh."""
    out = {}
    for name, mk in P1_MESHES.items():
        xy, tri = mk()
        out[f"{name}_xy"] = np.asarray(xy, dtype=np.float64)
        out[f"{name}_tri"] = np.asarray(tri, dtype=np.int32)
        for kind in ("laplace", "elastic"):
            ptr, col, val = ref.p1_assemble(xy, tri, kind, 210.0, 0.3)
            out[f"{name}_{kind}_ptr"], out[f"{name}_{kind}_col"], out[f"{name}_{kind}_val"] = ptr, col, val
    return out


def main():
    only = sys.argv[1:]
    if not ref.available():
        sys.exit("oracle/_ref/libLinA_ref.so is missing: run `make -C oracle ref` where the reference tree exists")
    if (not only or P1_FILE in only) and ref.fem2d_available():
        data = make_p1()
        path = os.path.join(HERE, f"{P1_FILE}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: " + ", ".join(f"{k[:-4]} {len(v)} entries" for k, v in data.items() if k.endswith("_val")))
    if not only or "spgemm" in only:
        data = make_spgemm()
        path = os.path.join(HERE, "spgemm.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: product with {len(data['c_col'])} entries")
    if not only or BATCH_FILE in only:
        data = make_batch()
        path = os.path.join(HERE, f"{BATCH_FILE}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: " + ", ".join(f"{k}={int(v)}" for k, v in data.items() if k.endswith("_it")))
    if not only or ILU_FILE in only:
        data = make_ilu()
        path = os.path.join(HERE, f"{ILU_FILE}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: " + ", ".join(f"{k}={int(v)}" for k, v in data.items() if k.endswith("_ok")))
    if not only or "fmg" in only:
        data = make_fmg()
        path = os.path.join(HERE, "fmg.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: {len(data)} full-multigrid results")
    if not only or SOLVERS_FILE in only:
        data = make_solvers()
        path = os.path.join(HERE, f"{SOLVERS_FILE}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: " + ", ".join(f"{k}={int(v)}" for k, v in data.items() if k.endswith("_it")))
    for name in ADJOINT_CASES:
        if only and name not in only:
            continue
        data = make_adjoint_case(name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: loss {float(data['loss']):.6e}, pcg iterations (target, forward, adjoint) {list(data['it'])}")
    for name in DIGEST_CASES:
        if name not in only:  # minutes of reference time: generated only when named
            continue
        data = make_digest_case(name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: sizes {list(data['sizes'])}, setup {float(data['ref_setup_s']):.1f} s, pcg iterations "
              + ", ".join(f"{k}={int(data[f'pcg_{k}_it'])}" for k in DIGEST_CASES[name][3]))
    for name in RN_DIGEST_CASES:
        if name not in only:
            continue
        data = make_rn_digest_case(name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: reflective Newton iterations {int(data['rn_umf_bicgstab_ilu_it'])}")
    for name in INDEF_CASES:
        if only and name not in only:
            continue
        data = make_indef_case(name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: reflective Newton iterations (negative-curvature events) "
              + ", ".join(f"{k}={int(data[f'rn_{k}_it'])} ({int(data[f'rn_{k}_negcurv'])})" for k in INDEF_SOLVERS))
    for name in RN_CASES:
        if only and name not in only:
            continue
        data = make_rn_case(name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: reflective Newton iterations "
              + ", ".join(f"{k}={int(data[f'rn_{k}_it'])}" for k in RN_SOLVERS))
    for name in CASES:
        if only and name not in only:
            continue
        data = make_case(name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: sizes {list(data['sizes'])}, pcg iterations "
              + ", ".join(f"{k}={int(data[f'pcg_{k}_it'])}" for k in SMOOTHERS))
    for name in SOLVE_CASES:
        if only and name not in only:
            continue
        data = make_solve_case(name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: sizes {list(data['sizes'])}, pcg iterations "
              + ", ".join(f"{k}={int(data[f'pcg_{k}_it'])}" for k in ("jacobi", "mcsor")))


if __name__ == "__main__":
    main()
