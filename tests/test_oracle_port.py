"""The CPU restatement (oracle/lina_port.c) against the reference's own outputs.

The golden files hold what the reference LinA computed (tests/golden/make_golden.py);
the restatement must reproduce V-cycles and complete pcg solves bit for bit.
"""
import numpy as np
import pytest

from oracle import port
from tests.conftest import golden_cases, load_golden

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
