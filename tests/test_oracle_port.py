"""The CPU restatement (oracle/lina_port.c, oracle/amg_setup_port.c) against the reference's own outputs.

The golden files hold what the reference LinA computed (tests/golden/make_golden.py);
the restatement must reproduce hierarchies, V-cycles and complete pcg solves bit for bit.
"""
import numpy as np
import pytest

from oracle import port, ref
from tests.conftest import golden_cases, load_golden, system_for
from tests.test_setup_parity import LIVE

SMOOTHERS = {"jacobi": (port.JACOBI, 0.6), "mcsor": (port.MC_SOR, 1.0), "refsor": (port.REF_SOR, 1.0)}


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
@pytest.mark.parametrize("smoother", list(SMOOTHERS))
def test_port_matches_reference(name, smoother):
    g = load_golden(name)
    kind, omega = SMOOTHERS[smoother]
    P = port.PortAMG(port.levels_from_golden(g), kind, omega, 2, 2)
    z = P.vcycle(g["vcycle_r"])
    assert np.array_equal(z, g[f"vcycle_{smoother}"])
    x, it, res = P.pcg(g["b"], 1e-8, 500, 0)
    assert it == int(g[f"pcg_{smoother}_it"])
    assert np.array_equal(x, g[f"pcg_{smoother}_x"])
    assert res == float(g[f"pcg_{smoother}_res"])


def _same(a, b):
    return (len(a[0]) == len(b[0]) and np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
            and np.array_equal(np.asarray(a[2]).view(np.int64), np.asarray(b[2]).view(np.int64)))


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
def test_port_setup_matches_reference_hierarchy(name):
    """The restated AMG_setup (oracle/amg_setup_port.c) gives the reference's hierarchy bit for bit,
    and the restated pcg on it the reference's solve."""
    g = load_golden(name)
    s = system_for(name)
    P = port.PortAMG.setup(s, int(g["depth"]), int(g["coarsening"]), 0.1, port.JACOBI, 0.6)
    assert P.sizes() == [int(v) for v in g["sizes"]]
    for l in range(int(g["depth"])):
        L = P.level(l)
        assert _same(L.A, (g[f"L{l}_A_ptr"], g[f"L{l}_A_col"], g[f"L{l}_A_val"])), f"A level {l}"
        if l > 0:
            assert np.array_equal(L.labels, g[f"L{l}_labels"]), f"labels level {l}"
            assert _same(L.P, (g[f"L{l}_P_ptr"], g[f"L{l}_P_col"], g[f"L{l}_P_val"])), f"P level {l}"
            assert _same(L.R, (g[f"L{l}_R_ptr"], g[f"L{l}_R_col"], g[f"L{l}_R_val"])), f"R level {l}"
    x, it, _ = P.pcg(g["b"], 1e-8, 500, 0)
    assert it == int(g["pcg_jacobi_it"])
    assert np.array_equal(x, g["pcg_jacobi_x"])


# the live cases of the library's own set-up test except the slowest reference run (aggressive at 129 x 129)
PORT_LIVE = [c for c in LIVE if c[0] != "elast129_aggr"]


@pytest.mark.skipif(not ref.available(), reason="reference library not built here (needs the reference tree)")
@pytest.mark.parametrize("case", PORT_LIVE, ids=[c[0] for c in PORT_LIVE])
def test_port_setup_matches_live_reference(case):
    _, factory, depth, coarsening = case
    s = factory()
    R = ref.hierarchy(s, depth, 2, 2, coarsening)
    P = port.PortAMG.setup(s, depth, coarsening)
    assert P.sizes() == R.sizes()
    for l in range(depth):
        a, b = R.level(l), P.level(l)
        assert _same(a.A, b.A), f"A level {l}"
        if l > 0:
            assert np.array_equal(a.labels, b.labels), f"labels level {l}"
            assert _same(a.P, b.P), f"P level {l}"
            assert _same(a.R, b.R), f"R level {l}"


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
def test_port_bicgstab_ilu_matches_reference(name):
    """The restated BiCGStab with ILU(0) (the damage workload's CPU baseline) reproduces the reference's
    BiCGStab_solve with its ILU(0) preconditioner bit for bit: iterations and solution."""
    g = load_golden(name)
    s = system_for(name)
    x, it, rel = port.bicgstab_ilu(s.indptr, s.indices, s.data, s.b, 1e-8, 1000)
    assert it == int(g["bicgstab_ilu_it"])
    assert np.array_equal(x, g["bicgstab_ilu_x"])
    assert rel <= 1e-8


@pytest.mark.skipif(not ref.available(), reason="reference library not built here (needs the reference tree)")
def test_port_bicgstab_ilu_matches_live_reference():
    """The same at a size beyond the goldens: the AT2 damage Hessian on a 129 x 129 mesh, whose
    factor rows mix short and long patterns."""
    from fem_gb300 import problems
    q = problems.at2_damage(129)
    xr, itr = ref.bicgstab_ilu(q, 1e-8, 1000)
    x, it, _ = port.bicgstab_ilu(q.indptr, q.indices, q.data, q.b, 1e-8, 1000)
    assert it == itr
    assert np.array_equal(x, xr)
