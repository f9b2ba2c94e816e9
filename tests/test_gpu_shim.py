"""The C++ header shim on the GPU: tests/cpp/shim_steps.cc drives the
reference's template API (ns::solver, mg::solver, ib::mac_grid /
ib::lagrangian_grid::interpolate) on the golden inputs, and its outputs match
the compiled reference's golden vectors at the FP64 tolerances."""
import os
import subprocess

import numpy as np
import pytest

from afmibins_gb300 import build, capi
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    capi.load()
    exe = str(tmp_path_factory.mktemp("shim") / "shim_steps")
    r = subprocess.run(["g++", "-std=c++14", "-O2", "-w", "-I", os.path.join(ROOT, "afmibins_gb300", "src"), "-I",
                        build.INCLUDE, os.path.join(ROOT, "tests", "cpp", "shim_steps.cc"), "-L", build.OUT_DIR,
                        "-lafmib", f"-Wl,-rpath,{build.OUT_DIR}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run(exe, cmd, arrays, tmp_path):
    fi, fo = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    np.concatenate([np.atleast_1d(np.asarray(a, dtype=np.float64)).ravel() for a in arrays]).tofile(fi)
    r = subprocess.run([exe, cmd, fi, fo], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return np.fromfile(fo, dtype=np.float64)


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_shim_ns_solver(driver, golden, tmp_path):
    d = golden("ns_16")
    r = _run(driver, "ns", [d["mu"], d["rho"], d["dt"], d["tol"], d["substeps"], d["u0"], d["v0"], d["w0"],
                            d["fx"], d["fy"], d["fz"]], tmp_path)
    N, NV, NXZ = 4096, 16 * 15 * 16, 256
    o = np.cumsum([0, N, NV, N, N, 4 * NXZ])
    assert rel(r[o[0]:o[1]], d["u"]) < 1e-10
    assert rel(r[o[1]:o[2]], d["v"]) < 1e-10
    assert rel(r[o[2]:o[3]], d["w"]) < 1e-10
    assert rel(r[o[4]:o[5]], d["walls"]) < 1e-10


def test_shim_mg_solver(driver, golden, tmp_path):
    d = golden("mg_test3_16")
    r = _run(driver, "mg", [d["tol"], d["rhs"]], tmp_path)
    x = r[1:]
    g = po.Grid(16, 16, 16, 16, channel=True)
    b = d["rhs"]
    res = (b - b.mean()) - po.lap_apply(g, x)
    assert np.sqrt(np.mean(res ** 2)) <= float(d["tol"])
    assert rel(x - x.mean(), d["x"] - d["x"].mean()) < 1e-9


def test_shim_ib_transfers(driver, golden, tmp_path):
    d = golden("ib_16")
    r = _run(driver, "ib", [d["X"].ravel(), d["vol"], d["F"][0], d["F"][1], d["F"][2], d["ue"], d["ve"], d["we"]],
             tmp_path)
    ns = d["spread"].size
    assert rel(r[:ns], d["spread"]) < 1e-13
    assert rel(r[ns:], d["interp"]) < 1e-13
