"""The drop-in LinA C API (include/*.h): a C caller compiled against the headers and
linked with the GPU library, and the row-list helpers against the reference."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from fem_gb300 import lina
from oracle import ref
from tests.conftest import ROOT, golden_cases, gpu_available, load_golden, system_for

DRIVER_SRC = os.path.join(ROOT, "tests", "c", "dropin_driver.c")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("drv") / "dropin_driver")
    libdir = os.path.dirname(lina.LIB_PATH)
    cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), DRIVER_SRC, "-o", exe,
           "-L", libdir, "-lLinA_gb300", f"-Wl,-rpath,{libdir}", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_driver_compiles_and_links_against_headers(driver):
    assert os.path.exists(driver)


def run_driver(driver, tmp_path, mode, s, depth, coarsening, smoother, omega):
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([s.n, s.nnz, s.dof, depth, coarsening, smoother], dtype=np.int32).tofile(f)
        np.array([omega], dtype=np.float64).tofile(f)
        np.ascontiguousarray(s.indptr, dtype=np.int32).tofile(f)
        np.ascontiguousarray(s.indices, dtype=np.int32).tofile(f)
        np.ascontiguousarray(s.data, dtype=np.float64).tofile(f)
        np.ascontiguousarray(s.b, dtype=np.float64).tofile(f)
    r = subprocess.run([driver, mode, str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = open(out, "rb").read()
    it = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    res = float(np.frombuffer(raw[4:12], dtype=np.float64)[0])
    x = np.frombuffer(raw[12:], dtype=np.float64)
    return it, res, x


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


gpu = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA device")]


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
@pytest.mark.parametrize("smoother,code,omega", [("jacobi", 2, 0.6), ("mcsor", 0, 1.0)])
@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_pcg_with_caller_vcycle_preconditioner(driver, tmp_path, name, smoother, code, omega):
    g = load_golden(name)
    s = system_for(name)
    it, res, x = run_driver(driver, tmp_path, "vcycle-pcg", s, int(g["depth"]), int(g["coarsening"]), code, omega)
    assert abs(it - int(g[f"pcg_{smoother}_it"])) <= 1
    assert rel(x, g[f"pcg_{smoother}_x"]) < 1e-9
    assert res == pytest.approx(float(g[f"pcg_{smoother}_res"]), rel=1e-3)


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
@pytest.mark.parametrize("smoother,code,omega", [("jacobi", 2, 0.6), ("mcsor", 0, 1.0)])
@pytest.mark.parametrize("mode", ["device-pcg", "device-pcg-clone"])
@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_pcg_with_library_vcycle_preconditioner(driver, tmp_path, name, smoother, code, omega, mode):
    """PCG_set_AMG_data + PCG_AMG_vcycle_precon: pcg on the device (device-pcg) or driven from the host
    with the preconditioner on the device (device-pcg-clone) reproduces the reference's pcg with a
    one-V-cycle zero-guess preconditioner: iterations within 1, solution within 1e-9."""
    g = load_golden(name)
    s = system_for(name)
    it, res, x = run_driver(driver, tmp_path, mode, s, int(g["depth"]), int(g["coarsening"]), code, omega)
    assert abs(it - int(g[f"pcg_{smoother}_it"])) <= 1
    assert rel(x, g[f"pcg_{smoother}_x"]) < 1e-9
    assert res == pytest.approx(float(g[f"pcg_{smoother}_res"]), rel=1e-3)


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_stock_amg_preconditioner(driver, tmp_path, name):
    """PCG_set_AMG_preconditioner: aggressive coarsening, warm-started V-cycles to 1e-2 (up to 100),
    multicolour SOR with omega 1.6 -- the reference run with the same smoother."""
    g = load_golden(name)
    s = system_for(name)
    it, res, x = run_driver(driver, tmp_path, "stock", s, int(g["depth"]), int(g["coarsening"]), 0, 1.6)
    assert abs(it - int(g["stock_it"])) <= 1
    assert rel(x, g["stock_x"]) < 1e-7


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_amg_solve_alone(driver, tmp_path, name):
    g = load_golden(name)
    s = system_for(name)
    it, res, x = run_driver(driver, tmp_path, "amgsolve", s, int(g["depth"]), int(g["coarsening"]), 2, 0.6)
    it_ref = int(g["amgsolve_jacobi_it"])
    assert abs(it - it_ref) <= max(1, it_ref // 20)
    xr = g["amgsolve_jacobi_x"]
    assert rel(x, xr) < (1e-6 if it_ref < 200 else 1e-3)


# ---------------------------------------------------------------- row-list helpers vs the reference
def _api(L):
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.sparse_zero.restype = vp
    L.sparse_zero.argtypes = [C.c_int]
    L.insert_sparse.restype = C.c_int
    L.insert_sparse.argtypes = [vp, C.c_double, C.c_int, C.c_int]
    L.sparse_product.restype = vp
    L.sparse_product.argtypes = [vp, vp]
    L.get_transpose.restype = vp
    L.get_transpose.argtypes = [vp, C.c_int]
    L.incomplete_LU_factorization.restype = C.c_int
    L.incomplete_LU_factorization.argtypes = [vp, vp, vp]
    L.Free_sparse.argtypes = [vp]
    return L


class SparseMatrix(C.Structure):
    _fields_ = [("Values", C.POINTER(C.POINTER(C.c_double))), ("Indices", C.POINTER(C.POINTER(C.c_int))),
                ("Len", C.POINTER(C.c_int)), ("size", C.c_int)]


def _read(ptr):
    m = C.cast(ptr, C.POINTER(SparseMatrix)).contents
    rows = []
    for i in range(m.size):
        rows.append([(m.Indices[i][k], m.Values[i][k]) for k in range(m.Len[i])])
    return rows


def _build(L, s):
    A = L.sparse_zero(s.n)
    for i in range(s.n):
        for p in range(s.indptr[i], s.indptr[i + 1]):
            L.insert_sparse(A, float(s.data[p]), i, int(s.indices[p]))
    return A


@pytest.mark.skipif(not ref.available(), reason="reference library not built here")
def test_row_list_helpers_match_reference():
    from fem_gb300 import problems
    s = problems.elasticity_p1(9)
    G = _api(C.CDLL(lina.LIB_PATH))
    R = _api(C.CDLL(ref.LIB_PATH))
    Ag, Ar = _build(G, s), _build(R, s)
    assert _read(Ag) == _read(Ar)
    assert _read(G.sparse_product(Ag, Ag)) == _read(R.sparse_product(Ar, Ar))
    assert _read(G.get_transpose(Ag, s.n)) == _read(R.get_transpose(Ar, s.n))
    Lg, Ug, Lr, Ur = G.sparse_zero(s.n), G.sparse_zero(s.n), R.sparse_zero(s.n), R.sparse_zero(s.n)
    assert G.incomplete_LU_factorization(Ag, Lg, Ug) == R.incomplete_LU_factorization(Ar, Lr, Ur) == 1
    assert _read(Lg) == _read(Lr) and _read(Ug) == _read(Ur)


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_spd_local_solver_matches_reference():
    """LinA_gpu_spd_solver (the library's AMG-PCG behind the slot signature int f(A, X, b)) on the 65 x 65
    elasticity system: the reference's tight solution; a second call with new values on the same pattern
    (the coarse levels recomputed) solves the scaled system."""
    g = load_golden("elast65_std_solve")
    s = system_for("elast65_std_solve")
    L = lina.dropin()
    L.LinA_gpu_spd_solver.restype = C.c_int
    L.LinA_gpu_spd_solver.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.AMG_set_deg_of_freedom.argtypes = [C.c_int]
    L.AMG_set_deg_of_freedom(2)
    A = lina.RowListView(s.indptr, s.indices, s.data)
    x = np.zeros(s.n)
    b = np.ascontiguousarray(s.b)
    assert L.LinA_gpu_spd_solver(A.ref, x.ctypes.data, b.ctypes.data) == 1
    assert rel(x, g["x_tight"]) < 1e-6
    A2 = lina.RowListView(s.indptr, s.indices, 2.0 * s.data)
    x2 = np.zeros(s.n)
    assert L.LinA_gpu_spd_solver(A2.ref, x2.ctypes.data, b.ctypes.data) == 1
    assert rel(x2, 0.5 * g["x_tight"]) < 1e-6
