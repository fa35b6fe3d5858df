"""The C-ABI library builds, loads and exports every symbol include/*.h declares.

CPU-only: loads the shared object and inspects its symbol table; no compute
call is made (there is no GPU here).
"""
import ctypes
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        with open(h) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, re.M):
            name = m.group(1)
            if name not in ("if", "defined"):
                names.add(name)
    return names


@pytest.fixture(scope="module")
def libpath():
    from enlightning_gb300 import build
    return build.build()


def test_header_declares_dropin_symbols():
    names = declared_symbols()
    for s in ("rhs_", "runge_kutta_", "update_state_", "tag_cells_"):
        assert s in names


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = sorted(declared_symbols() - exported)
    assert not missing, f"declared but not exported: {missing}"


def test_library_loads_without_gpu(libpath):
    lib = ctypes.CDLL(libpath)
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_binding_signatures_cover_header():
    from enlightning_gb300 import _lib
    missing = sorted(declared_symbols() - set(_lib.SIGNATURES))
    assert not missing, f"no ctypes signature for {missing}"
