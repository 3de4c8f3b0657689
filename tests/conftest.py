"""Shared test setup: markers, builds of the library and of the CPU oracle, fixtures."""
import glob
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def _ensure_built():
    from fem_gb300 import build as B
    B.build()
    port = os.path.join(ROOT, "oracle", "_build", "liblina_port.so")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    assert os.path.exists(port)


_ensure_built()


def gpu_available() -> bool:
    from fem_gb300 import lina
    try:
        return lina.lib().lina_gpu_device_count() > 0
    except Exception:
        return False


def golden_cases(kind="hierarchy"):
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        g = np.load(f)
        if "digest" not in g.files and "L0_A_ptr" not in g.files:
            continue  # not a linear-system fixture (reflective Newton quadratics)
        if "sample_index" in g.files:
            continue  # a configuration-size digest (tests/test_config_parity.py), without the system itself
        has_h = "L0_A_ptr" in g.files
        if (kind == "hierarchy") == has_h:
            out.append(os.path.basename(f)[:-4])
    return out


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def system_for(name):
    """The exact input system of a golden case, as the reference received it.

    The stored arrays are used rather than a regeneration because numpy's
    transcendental functions may differ in the last bit between x86 and Arm
    hosts (the damage field uses exp); tests/test_problems.py checks that the
    generator reproduces the stored input.
    """
    from fem_gb300 import problems
    g = load_golden(name)
    return problems.CSRSystem(int(g["n"]), g["indptr"], g["indices"], g["data"], g["b"], dof=int(g["dof"]),
                              meta={"golden": name})


def regenerate(name):
    from tests.golden.make_golden import CASES, SOLVE_CASES
    factory = (CASES.get(name) or SOLVE_CASES.get(name))[0]
    return factory()
