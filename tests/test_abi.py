"""The C-ABI library loads and exports every function its headers declare (no GPU needed)."""
import os
import re
import subprocess

from fem_gb300 import lina
from tests.conftest import ROOT

INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for f in sorted(os.listdir(INCLUDE)):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        text = re.sub(r"#[^\n]*", "", text)
        for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", text):
            name = m.group(1)
            before = text[max(0, m.start() - 80):m.start()]
            if "typedef" in before.split(";")[-1]:
                continue
            if name in {"if", "while", "for", "return", "sizeof", "int", "void", "double", "float", "char", "long",
                        "unsigned"}:
                continue
            names.add(name)
    return names


def exported_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", lina.LIB_PATH], capture_output=True, text=True, check=True)
    return {line.split()[-1] for line in out.stdout.splitlines() if line.strip()}


def test_library_loads():
    assert lina.lib() is not None


def test_every_declared_symbol_is_exported():
    missing = sorted(declared_functions() - exported_symbols())
    assert not missing, f"declared in include/*.h but not exported: {missing}"
