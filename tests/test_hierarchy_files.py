"""Hierarchy files (lina_gpu_amg_save / lina_gpu_amg_load) and the drop-in write_sparse /
read_sparse (LinA/linear_algebra.c:832-869).

A saved and reloaded hierarchy must equal the original level by level (patterns, values, labels),
and solve exactly as it did; the matrix files are the reference's binary format, checked against
the reference's own reader and writer where the reference library is built.
"""
import ctypes as C

import numpy as np
import pytest

from fem_gb300 import lina, problems
from oracle import ref
from tests.conftest import golden_cases, gpu_available, load_golden, system_for


class SparseMatrix(C.Structure):
    _fields_ = [("Values", C.POINTER(C.POINTER(C.c_double))), ("Indices", C.POINTER(C.POINTER(C.c_int))),
                ("Len", C.POINTER(C.c_int)), ("size", C.c_int)]


def same(a, b):
    return (len(a[0]) == len(b[0]) and np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
            and np.array_equal(np.asarray(a[2]).view(np.int64), np.asarray(b[2]).view(np.int64)))


def assert_same_hierarchy(a, b):
    assert a.depth == b.depth and a.sizes() == b.sizes()
    for l in range(a.depth):
        x, y = a.level(l), b.level(l)
        assert same(x.A, y.A), f"A level {l}"
        if l > 0:
            assert np.array_equal(x.labels, y.labels), f"labels level {l}"
            assert same(x.P, y.P) and same(x.R, y.R), f"P/R level {l}"


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
def test_host_round_trip(name, tmp_path):
    g = load_golden(name)
    s = system_for(name)
    a = lina.AMG.from_system(s, host_only=True, depth=int(g["depth"]), coarsening=int(g["coarsening"]))
    a.save(tmp_path / "h")
    b = lina.AMG.load(tmp_path / "h", host_only=True)
    assert_same_hierarchy(a, b)


def test_load_rejects_missing_or_damaged_files(tmp_path):
    with pytest.raises(lina.LinaError):
        lina.AMG.load(tmp_path / "nothing", host_only=True)
    s = problems.poisson_p1(17, seed=0)
    a = lina.AMG.from_system(s, host_only=True, depth=3)
    a.save(tmp_path / "h")
    (tmp_path / "h" / "L1_P").write_bytes(b"\x05\x00")
    with pytest.raises(lina.LinaError):
        lina.AMG.load(tmp_path / "h", host_only=True)


def _write_with(libfn, csr, directory, name):
    ptr, col, val = csr
    n = len(ptr) - 1
    lens = np.diff(ptr).astype(np.int32)
    rows_c = [np.ascontiguousarray(col[ptr[i]:ptr[i + 1]], dtype=np.int32) for i in range(n)]
    rows_v = [np.ascontiguousarray(val[ptr[i]:ptr[i + 1]], dtype=np.float64) for i in range(n)]
    A = SparseMatrix()
    A.size = n
    A.Len = lens.ctypes.data_as(C.POINTER(C.c_int))
    ip = (C.POINTER(C.c_int) * n)(*[r.ctypes.data_as(C.POINTER(C.c_int)) for r in rows_c])
    vp = (C.POINTER(C.c_double) * n)(*[r.ctypes.data_as(C.POINTER(C.c_double)) for r in rows_v])
    A.Indices = C.cast(ip, C.POINTER(C.POINTER(C.c_int)))
    A.Values = C.cast(vp, C.POINTER(C.POINTER(C.c_double)))
    libfn.restype = C.c_int
    libfn.argtypes = [C.POINTER(SparseMatrix), C.c_char_p, C.c_char_p]
    assert libfn(C.byref(A), str(directory).encode(), name.encode()) == 1


def _read_with(libfn, directory, name):
    libfn.restype = C.POINTER(SparseMatrix)
    libfn.argtypes = [C.c_char_p, C.c_char_p]
    p = libfn(str(directory).encode(), name.encode())
    assert p
    A = p.contents
    ptr, col, val = [0], [], []
    for i in range(A.size):
        k = A.Len[i]
        col.extend(A.Indices[i][j] for j in range(k))
        val.extend(A.Values[i][j] for j in range(k))
        ptr.append(ptr[-1] + k)
    return np.array(ptr), np.array(col), np.array(val)


def test_dropin_write_read_round_trip(tmp_path):
    s = problems.elasticity_p1(9)
    csr = (s.indptr, s.indices, s.data)
    _write_with(lina.lib().write_sparse, csr, tmp_path, "m.bin")
    # the file layout: n, Len[n], indices row by row, values row by row
    raw = (tmp_path / "m.bin").read_bytes()
    n = s.n
    assert np.frombuffer(raw[:4], np.int32)[0] == n
    assert np.array_equal(np.frombuffer(raw[4:4 + 4 * n], np.int32), np.diff(s.indptr))
    assert len(raw) == 4 + 4 * n + 12 * s.nnz
    assert same(_read_with(lina.lib().read_sparse, tmp_path, "m.bin"), csr)


@pytest.mark.skipif(not ref.available(), reason="reference library not built here (needs the reference tree)")
def test_files_interchange_with_reference(tmp_path):
    """The reference reads the library's files and the library reads the reference's."""
    s = problems.poisson_p1(17, seed=1)
    csr = (s.indptr, s.indices, s.data)
    _write_with(lina.lib().write_sparse, csr, tmp_path, "ours.bin")
    assert same(_read_with(ref.lib().read_sparse, tmp_path, "ours.bin"), csr)
    _write_with(ref.lib().write_sparse, csr, tmp_path, "theirs.bin")
    assert same(_read_with(lina.lib().read_sparse, tmp_path, "theirs.bin"), csr)
    assert (tmp_path / "ours.bin").read_bytes() == (tmp_path / "theirs.bin").read_bytes()
    # a saved hierarchy level is a reference matrix file
    a = lina.AMG.from_system(s, host_only=True, depth=3)
    a.save(tmp_path / "h")
    L = a.level(1)
    assert same(_read_with(ref.lib().read_sparse, tmp_path / "h", "L1_P"), L.P)


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
@pytest.mark.parametrize("name", golden_cases("hierarchy"))
@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
def test_loaded_hierarchy_solves_identically(name, precision, tmp_path):
    g = load_golden(name)
    s = system_for(name)
    opts = dict(smoother=lina.SMOOTHER_MC_SOR, omega=1.0, precision=precision)
    a = lina.AMG.from_system(s, depth=int(g["depth"]), coarsening=int(g["coarsening"]), **opts)
    a.save(tmp_path / "h")
    b = lina.AMG.load(tmp_path / "h", **opts)
    assert_same_hierarchy(a, b)
    x1, i1 = a.pcg(s.b, tol=1e-8, max_iter=500)
    x2, i2 = b.pcg(s.b, tol=1e-8, max_iter=500)
    assert i1.status == 0 and i1.iterations == i2.iterations
    assert np.array_equal(x1, x2)
