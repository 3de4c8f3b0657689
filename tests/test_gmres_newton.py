"""gmres, Newton_solver and active_set_solver against the reference (tests/golden/solvers.npz).

A C caller (tests/c/solvers_driver.c) drives the drop-in API the way FEM2D/FEM.c and
Crack/crack.c do.  gmres and the ILU-GMRES Newton steps run on the GPU; the sparse-LU Newton
steps and the active-set loop with a caller-supplied dense KKT solver are host code and are
checked on the CPU as well.
"""
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

from fem_gb300 import lina, problems
from tests.conftest import ROOT

DRIVER_SRC = os.path.join(ROOT, "tests", "c", "solvers_driver.c")
GOLDEN = os.path.join(ROOT, "tests", "golden", "solvers.npz")
SOL_TOL = 1e-7  # relative error of solutions against the reference


def load():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def it_ok(it, it_ref):
    return abs(it - it_ref) <= max(1, int(np.ceil(0.1 * it_ref)))


SYSTEMS = {"poisson33": lambda: problems.poisson_p1(33, seed=0), "elast17": lambda: problems.elasticity_p1(17)}


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("solvers") / "solvers_driver")
    libdir = os.path.dirname(lina.LIB_PATH)
    cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), DRIVER_SRC, "-o", exe,
           "-L", libdir, "-lLinA_gb300", f"-Wl,-rpath,{libdir}", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def run(driver, tmp_path, mode, s, ints, dbls, b=None, x0=None, lower=None, upper=None):
    inp, out = tmp_path / f"{mode}.in", tmp_path / f"{mode}.out"
    n = s.n
    with open(inp, "wb") as f:
        np.array([n, s.nnz] + list(ints), dtype=np.int32).tofile(f)
        np.array(dbls, dtype=np.float64).tofile(f)
        np.ascontiguousarray(s.indptr, dtype=np.int32).tofile(f)
        np.ascontiguousarray(s.indices, dtype=np.int32).tofile(f)
        np.ascontiguousarray(s.data, dtype=np.float64).tofile(f)
        for v in (s.b if b is None else b, np.zeros(n) if x0 is None else x0,
                  np.full(n, -1e300) if lower is None else lower, np.full(n, 1e300) if upper is None else upper):
            np.ascontiguousarray(v, dtype=np.float64).tofile(f)
    r = subprocess.run([driver, mode, str(inp), str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    raw = out.read_bytes()
    ints_out = np.frombuffer(raw[:12], dtype=np.int32)
    d = float(np.frombuffer(raw[12:20], dtype=np.float64)[0])
    x = np.frombuffer(raw[20:], dtype=np.float64).copy()
    return ints_out, d, x


def test_solvers_driver_compiles(driver):
    assert os.path.exists(driver)


def test_reference_gmres_iterates_solve_the_system():
    """Pins the oracle: x = ILU^-1 y of each stored reference run meets its tolerance."""
    g = load()
    for name, make in SYSTEMS.items():
        s = make()
        A = sp.csr_matrix((s.data, s.indices, s.indptr), shape=(s.n, s.n))
        for check in (0, 1):
            key = f"gmres_{name}_{check}"
            assert int(g[key + "_rc"]) == 0
            x = g[key + "_x"]
            assert np.linalg.norm(s.b - A @ x) / np.linalg.norm(s.b) <= 10 * float(g[key + "_tol"])


def gpu_ilu_solve(s):
    """x = U^-1 L^-1 y with the library's device ILU(0) (its application is checked against the
    reference's in test_gpu_solve)."""
    ilu = lina.ILU(s.n, s.indptr, s.indices, s.data)
    return ilu.apply


@pytest.mark.parametrize("mode", [0])
def test_newton_sparse_lu_matches_reference(driver, tmp_path, mode):
    """SMALL_SYSTEM Newton steps (sparse LU on the host)."""
    g = load()
    s = problems.poisson_p1(17, seed=2)
    ints, _, x = run(driver, tmp_path, "newton", s, [mode, 20, 50], [1e-10, 50.0], b=g["newton_B"])
    it_ref = int(g[f"newton_{mode}_it"])
    assert it_ok(int(ints[0]), it_ref), (ints[0], it_ref)
    assert rel(x, g[f"newton_{mode}_x"]) <= SOL_TOL


def test_active_set_matches_reference(driver, tmp_path):
    g = load()
    s = problems.poisson_p1(17, seed=1)
    ints, _, x = run(driver, tmp_path, "active", s, [100, 0, 0], [0.0, 0.0], lower=g["active_lower"],
                     upper=g["active_upper"])
    assert int(ints[0]) == int(g["active_it"]) and int(ints[1]) == int(g["active_size"])
    assert rel(x, g["active_x"]) <= SOL_TOL
    assert x.min() >= g["active_lower"].min() - 1e-9 and x.max() <= g["active_upper"].max() + 1e-9


@pytest.mark.gpu
def test_active_set_with_gpu_kkt_solver_matches_reference(driver, tmp_path):
    """active_set_solver with LinA_gpu_general_solver (GMRES + ILU(0) on the device) solving its KKT
    systems, in the slot crack.c fills with its UMFPACK wrapper: the reference's active set and solution."""
    g = load()
    s = problems.poisson_p1(17, seed=1)
    ints, _, x = run(driver, tmp_path, "active-gpu", s, [100, 0, 0], [0.0, 0.0], lower=g["active_lower"],
                     upper=g["active_upper"])
    assert int(ints[0]) == int(g["active_it"]) and int(ints[1]) == int(g["active_size"])
    assert rel(x, g["active_x"]) <= SOL_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("check", [0, 1])
@pytest.mark.parametrize("mode", ["gmres", "gmres-host"])
def test_gmres_matches_reference(driver, tmp_path, name, check, mode):
    g = load()
    s = SYSTEMS[name]()
    key = f"gmres_{name}_{check}"
    ints, prec, y = run(driver, tmp_path, mode, s, [20, 1000, check], [float(g[key + "_tol"]), 0.0])
    it, rc = int(ints[0]), int(ints[1])
    assert rc == int(g[key + "_rc"]) == 0
    assert it_ok(it, int(g[key + "_it"])), (it, int(g[key + "_it"]))
    assert prec <= float(g[key + "_tol"])
    assert rel(gpu_ilu_solve(s)(y), g[key + "_x"]) <= SOL_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(SYSTEMS))
def test_gmres_c_abi(name):
    """lina_gpu_gmres with the device ILU(0) as right preconditioner, x = B_r y returned."""
    g = load()
    s = SYSTEMS[name]()
    key = f"gmres_{name}_0"
    M = lina.Matrix(s.n, s.indptr, s.indices, s.data)
    ilu = lina.ILU(s.n, s.indptr, s.indices, s.data)
    x, info = lina.gmres(M, s.b, ilu=ilu, tol=float(g[key + "_tol"]), i_max=20, max_iter=1000, apply_precon=True)
    assert info.status == 0 and it_ok(info.iterations, int(g[key + "_it"]))
    assert rel(x, g[key + "_x"]) <= SOL_TOL


@pytest.mark.gpu
def test_newton_gmres_matches_reference(driver, tmp_path):
    """LARGE_SYSTEM Newton steps: ILU(0)-preconditioned GMRES on the GPU."""
    g = load()
    s = problems.poisson_p1(17, seed=2)
    ints, _, x = run(driver, tmp_path, "newton", s, [1, 20, 50], [1e-10, 50.0], b=g["newton_B"])
    it_ref = int(g["newton_1_it"])
    assert it_ok(int(ints[0]), it_ref), (ints[0], it_ref)
    assert rel(x, g["newton_1_x"]) <= SOL_TOL
