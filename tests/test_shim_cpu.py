"""The C++ header shim (afmibins_gb300/src/{dt,alg,mg,ns,ib}) keeps the
reference's template API: the shim driver compiles against it, and — where the
reference sources are present — the reference's own seven test programs
compile and link unchanged against the shim and libafmib.so. No GPU calls."""
import os
import subprocess

import pytest

from afmibins_gb300 import build, capi
from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "afmibins_gb300", "src")


def _cxx(src, out, extra=()):
    capi.load()
    cmd = ["g++", "-std=c++14", "-O1", "-w", "-I", SHIM, "-I", build.INCLUDE, src, "-L", build.OUT_DIR, "-lafmib",
           f"-Wl,-rpath,{build.OUT_DIR}", "-o", out, *extra]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_shim_driver_compiles(tmp_path):
    r = _cxx(os.path.join(ROOT, "tests", "cpp", "shim_steps.cc"), str(tmp_path / "shim_steps"))
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(not po.reference_available(), reason="reference sources not present")
@pytest.mark.parametrize("prog", ["ns_test", "ib_ns_test", "ib_test", "mg_test", "mg_test2", "mg_test3", "restr_test"])
def test_reference_programs_compile_against_shim(tmp_path, prog):
    src = os.path.join(po.REFERENCE_SRC, "test", prog + ".cc")
    r = _cxx(src, str(tmp_path / prog))
    assert r.returncode == 0, r.stderr
