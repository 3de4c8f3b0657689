"""Reflective Newton (LinA/reflective_newton.c) through the drop-in C API.

A C caller (tests/c/rn_driver.c) sets a bound-constrained quadratic up the way
Crack/crack.c does and runs ``reflective_newton`` of the GPU library with three
local solvers; the minimiser and the Newton iteration count are compared with
what the reference computed on the same quadratic (tests/golden/damage*_rn.npz,
made by tests/golden/make_golden.py).
"""
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

from fem_gb300 import lina, problems
from tests.conftest import ROOT, gpu_available

DRIVER_SRC = os.path.join(ROOT, "tests", "c", "rn_driver.c")
GOLDEN = os.path.join(ROOT, "tests", "golden")
RN_FACTORIES = {"damage65_rn": lambda: problems.damage_qp(65), "damage129_rn": lambda: problems.damage_qp(129),
                "at2_65_rn": lambda: problems.at2_damage(65)}
RN_CASES = list(RN_FACTORIES)

# The minimiser is unique (H is SPD); the iterates differ from the reference's
# only through the inner solves, which stop at a relative residual of 1e-8.
X_TOL = 1e-6
# Newton iterations: within 10 % of the reference, at least one either way
def it_slack(it_ref):
    return max(1, int(np.ceil(0.1 * it_ref)))


def load(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("rn") / "rn_driver")
    libdir = os.path.dirname(lina.LIB_PATH)
    cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), DRIVER_SRC, "-o", exe,
           "-L", libdir, "-lLinA_gb300", f"-Wl,-rpath,{libdir}", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_rn_driver_compiles_and_links(driver):
    assert os.path.exists(driver)


@pytest.mark.parametrize("name", RN_CASES)
def test_golden_inputs_regenerate(name):
    g = load(name)
    q = RN_FACTORIES[name]()
    assert np.array_equal(q.indptr, g["indptr"]) and np.array_equal(q.indices, g["indices"])
    np.testing.assert_allclose(q.data, g["data"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(q.b, g["b"], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(q.meta["lower"], g["lower"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("name", RN_CASES)
@pytest.mark.parametrize("solver", ["umf_bicgstab_ilu", "pcg_ilu"])
def test_reference_minimiser_satisfies_kkt(name, solver):
    """The stored reference result is a box-constrained minimiser: feasible, with the
    scaled gradient of the reflective Newton method (gradient times the distance to the
    bound it points to) vanishing, and gradients pointing outward at active bounds."""
    g = load(name)
    n = int(g["n"])
    H = sp.csr_matrix((g["data"], g["indices"], g["indptr"]), shape=(n, n))
    x = g[f"rn_{solver}_x"]
    lo, up = g["lower"], g["upper"]
    assert np.all(x >= lo) and np.all(x <= up)
    grad = H @ x + g["b"]
    scale = np.abs(g["b"]).max()
    at_lo = np.abs(x - lo) < 1e-9
    at_up = np.abs(x - up) < 1e-9
    free = ~(at_lo | at_up)
    assert at_lo.any() and free.any()
    dist = np.minimum(np.where(grad < 0, up - x, x - lo), 1.0)
    # the reference stops on a relative functional decrease of 1e-8, not on this measure
    assert (np.abs(grad) * dist).max() < 1e-6 * scale
    assert grad[at_lo].min() > -1e-5 * scale
    if at_up.any():
        assert grad[at_up].max() < 1e-5 * scale


def run_rn(driver, tmp_path, mode, g, max_iter=50, eps=1e-8, bi_eps=1e-8):
    inp, out = tmp_path / f"rn_{mode}.in", tmp_path / f"rn_{mode}.out"
    n = int(g["n"])
    with open(inp, "wb") as f:
        np.array([n, len(g["indices"]), max_iter], dtype=np.int32).tofile(f)
        np.array([eps, bi_eps], dtype=np.float64).tofile(f)
        np.ascontiguousarray(g["indptr"], dtype=np.int32).tofile(f)
        np.ascontiguousarray(g["indices"], dtype=np.int32).tofile(f)
        for k in ("data", "b", "lower", "upper", "x0"):
            np.ascontiguousarray(g[k], dtype=np.float64).tofile(f)
    r = subprocess.run([driver, mode, str(inp), str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    raw = out.read_bytes()
    it = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    x = np.frombuffer(raw[4:], dtype=np.float64).copy()
    assert x.size == n
    return it, x


@pytest.mark.gpu
@pytest.mark.parametrize("name", RN_CASES)
@pytest.mark.parametrize("mode,ref_solver", [("gpu", "umf_bicgstab_ilu"), ("umf", "umf_bicgstab_ilu"),
                                             ("pcg", "pcg_ilu"), ("spd", "umf_bicgstab_ilu")])
def test_reflective_newton_matches_reference(driver, tmp_path, name, mode, ref_solver):
    g = load(name)
    it, x = run_rn(driver, tmp_path, mode, g)
    x_ref = g[f"rn_{ref_solver}_x"]
    it_ref = int(g[f"rn_{ref_solver}_it"])
    assert it > 0
    assert abs(it - it_ref) <= it_slack(it_ref), (it, it_ref)
    assert np.all(x >= g["lower"]) and np.all(x <= g["upper"])
    err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
    assert err <= X_TOL, err
    # the active sets agree (an unknown within 1e-6 of a bound may be snapped on one side only)
    for bound in ("lower", "upper"):
        mismatch = np.count_nonzero((np.abs(x - g[bound]) < 1e-9) != (np.abs(x_ref - g[bound]) < 1e-9))
        assert mismatch <= 2, (bound, mismatch)


@pytest.mark.gpu
@pytest.mark.parametrize("name", RN_CASES)
def test_csr_entry_point_matches_reference(name):
    """lina_gpu_reflective_newton_csr (the drop-in set-up done by the library) with the device
    BiCGStab + ILU(0) local solver against the reference's minimiser."""
    g = load(name)
    q = RN_FACTORIES[name]()
    x, it = lina.reflective_newton(q, g["lower"], g["upper"], g["x0"])
    x_ref = g["rn_umf_bicgstab_ilu_x"]
    it_ref = int(g["rn_umf_bicgstab_ilu_it"])
    assert abs(it - it_ref) <= it_slack(it_ref), (it, it_ref)
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) <= X_TOL


def _neg_curv_events(tmp_path):
    """number_neg_curv of the library's RN statistics, read through print_RN_statistics."""
    import ctypes as C
    libc = C.CDLL(None)
    libc.fopen.restype, libc.fopen.argtypes = C.c_void_p, [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    L = lina.lib()
    L.print_RN_statistics.argtypes = [C.c_void_p]
    path = str(tmp_path / "rnstat.txt")
    f = libc.fopen(path.encode(), b"w")
    L.print_RN_statistics(f)
    libc.fclose(f)
    for line in open(path):
        if line.startswith("number of neg. curvature events:"):
            return int(line.split(":")[1])
    return -1


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
@pytest.mark.parametrize("solver,ref_name", [(4, "cholesky"), (lina.RN_GPU_BICGSTAB_ILU, "umf_bicgstab_ilu")])
def test_indefinite_quadratic_matches_reference(solver, ref_name, tmp_path):
    """An indefinite Hessian (grid Laplacian minus 0.5 I, tests/golden/indef17_rn.npz): with the complete
    Cholesky local solver (RN_CHOLESKY) the scaled matrix is reported INDEFINITE and the step takes the
    direction of negative curvature found by the shifted power iteration, as in the reference (whose
    start vector is drawn with the same seed); BiCGStab + ILU(0) solves the indefinite systems as the
    reference's BiCGStab did.  Minimiser within 1e-6, Newton steps within 10 %, the same number of
    negative-curvature events."""
    g = load("indef17_rn")
    q = problems.indefinite_qp(17)
    assert np.array_equal(q.data, g["data"]) and np.array_equal(q.b, g["b"])
    lina.lib().RN_init_statistics()
    x, it = lina.reflective_newton(q, g["lower"], g["upper"], g["x0"], solver=solver)
    it_ref = int(g[f"rn_{ref_name}_it"])
    assert abs(it - it_ref) <= it_slack(it_ref), (it, it_ref)
    assert np.max(np.abs(x - g[f"rn_{ref_name}_x"])) <= X_TOL
    assert _neg_curv_events(tmp_path) == int(g[f"rn_{ref_name}_negcurv"])
