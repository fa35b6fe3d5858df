"""Build the reference's own boundary routines into oracle/_ref (test infrastructure).

The reference's absorbing envelope (enlightning::setAbsorbingBoundaryConditions,
enlightning.C:634-786) and physical-boundary ghost fill
(enlightning::setPhysicalBoundaryConditions, enlightning.C:790-1013) are plain
pointer loops over SAMRAI cell data.  This recipe reads the reference's
enlightning.C where it lies, takes the text of those two member functions
unchanged (located by their signatures, ended by brace matching), and compiles
it after ``samrai_stub.h`` (stand-ins for the SAMRAI types they use) and before
``ref_bc_driver.cpp`` (C entry points ref_absorb / ref_phys_bc with the
oracle's argument lists).  The source goes to g++ on standard input, so no copy
of it is written anywhere; the only output is ``oracle/_ref/libenl_bc_ref.so``.

Usage: python oracle/ref_bc.py <reference root>
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libenl_bc_ref.so")
FUNCS = ("void enlightning::setAbsorbingBoundaryConditions",
         "void enlightning::setPhysicalBoundaryConditions")


def extract(text: str, signature: str) -> str:
    """The definition that starts at `signature`, through its closing brace."""
    start = text.index(signature)
    depth, k = 0, text.index("{", start)
    while True:
        ch = text[k]
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth -= 1
            if depth == 0:
                return text[start:k + 1]
        k += 1


def build(reference_root: str, force: bool = False) -> str:
    src = os.path.join(reference_root, "enlightning.C")
    os.makedirs(OUT, exist_ok=True)
    deps = [src, os.path.join(HERE, "samrai_stub.h"), os.path.join(HERE, "ref_bc_driver.cpp"), __file__]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    with open(src) as f:
        text = f.read()
    parts = ['#include "samrai_stub.h"', '#line 1 "enlightning.C (extracted)"']
    parts += [extract(text, sig) for sig in FUNCS]
    with open(os.path.join(HERE, "ref_bc_driver.cpp")) as f:
        parts.append('#line 1 "ref_bc_driver.cpp"\n' + f.read())
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-I", HERE, "-x", "c++", "-", "-o", tmp]
    subprocess.run(cmd, input="\n".join(parts).encode(), check=True)
    os.replace(tmp, LIB)
    return LIB


def load(path: str = LIB):
    L = C.CDLL(path)
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    i, d = C.c_int, C.c_double
    L.ref_absorb.argtypes = [i, i, i, i, i, i, dp, dp, dp, dp, ip, d, d, d, d, dp, dp, dp]
    L.ref_absorb.restype = None
    L.ref_phys_bc.argtypes = [i, i, i, i, i, i, ip, ip, i, i, dp, dp, dp, dp]
    L.ref_phys_bc.restype = None
    return L


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/ref_bc.py <reference root>")
    print(build(sys.argv[1], force=True))
