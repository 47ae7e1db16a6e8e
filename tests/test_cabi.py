"""The C-ABI library loads, exports every symbol include/Spirit_gb300.h declares (and nothing
undeclared), and the header compiles as C.  No device compute: these run on any host."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "Spirit_gb300.h")
LIB = os.path.join(ROOT, "spirit_gb300", "libspirit_gb300.so")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", " ", txt, flags=re.S)
    names = set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt))
    return {n for n in names if n[0].isupper() or n == "free_run_info"} - {"SPIRIT_GB300_H"}


def exported():
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True, check=True).stdout
    return {l.split()[2] for l in out.splitlines() if len(l.split()) == 3 and l.split()[1] == "T"
            and not l.split()[2].startswith("_Z")}


@pytest.fixture(scope="module", autouse=True)
def built():
    if not os.path.exists(LIB):
        from spirit_gb300 import build
        build.build()


def test_library_loads():
    ctypes.CDLL(LIB)


def test_every_declared_symbol_is_exported():
    missing = declared() - exported()
    assert not missing, sorted(missing)


def test_every_exported_symbol_is_declared():
    extra = exported() - declared()
    assert not extra, sorted(extra)


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "Spirit_gb300.h"\nint main(void){ return Solver_Heun; }\n')
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-fsyntax-only", "-I", os.path.dirname(HEADER), str(src)],
                   check=True)
