"""Snapshot files without a GPU: the library's writer (snapshot_io.h, built for
the host) against the Python reader (afmibins_gb300/snapshot.py), and the
C++ reader's checks on damaged files."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from afmibins_gb300 import build, snapshot

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("snap") / "libsnap.so"
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(build.PKG, "csrc"),
                    os.path.join(HERE, "cpp", "snapshot_host.cc"), "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    L.afmib_test_snapshot_write.argtypes = [ctypes.c_char_p]
    L.afmib_test_snapshot_read.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    return L


def _read_c(lib, path):
    err = ctypes.create_string_buffer(128)
    n, su = ctypes.c_int(), ctypes.c_double()
    rc = lib.afmib_test_snapshot_read(os.fsencode(path), err, 128, ctypes.byref(n), ctypes.byref(su))
    return rc, err.value.decode(), n.value, su.value


def test_library_writer_python_reader(lib, tmp_path):
    p = tmp_path / "a.snap"
    assert lib.afmib_test_snapshot_write(os.fsencode(str(p))) == 0
    sec = snapshot.read(str(p))
    h = sec["header"]
    assert (h["nx"], h["ny"], h["nz"], h["n"], h["bc"], h["precision"], h["half"]) == (4, 3, 2, 4, 1, 1, 1)
    assert h["substeps"] == 7 and h["mg_rho"] == 0.125
    i = np.arange(24)
    np.testing.assert_array_equal(sec["u"], 0.5 + i)
    np.testing.assert_array_equal(sec["v"], -0.25 * i)
    np.testing.assert_array_equal(sec["phi_prev0"], 1e-3 * i * i - 1.0)
    assert sec["X"].shape == (15,) and sec["nstart"].dtype == np.int32
    np.testing.assert_array_equal(sec["nidx"][:4], [4, 1, 0, 2])
    counts = snapshot.sections(str(p))
    assert counts["walls"][1] == 32 and "phi_prev1" not in counts
    np.testing.assert_array_equal(sec["wallgrad"], -0.5 * np.arange(48))
    rc, err, n, su = _read_c(lib, str(p))
    assert rc == 0 and err == "" and n == 11 and su == float(np.sum(0.5 + i))


def test_damaged_files_are_rejected(lib, tmp_path):
    p = tmp_path / "a.snap"
    assert lib.afmib_test_snapshot_write(os.fsencode(str(p))) == 0
    raw = p.read_bytes()
    cases = {"not a snapshot file": b"XXXXXXXX" + raw[8:], "unsupported snapshot version": raw[:8] + b"\x02" + raw[9:],
             "truncated snapshot": raw[:-7], "bad section type": raw[:64 + 16] + b"\x09" + raw[64 + 17:]}
    for want, data in cases.items():
        q = tmp_path / "bad.snap"
        q.write_bytes(data)
        rc, err, _, _ = _read_c(lib, str(q))
        assert rc == 1 and err == want, (want, err)
        with pytest.raises(ValueError):
            snapshot.read(str(q))
    rc, err, _, _ = _read_c(lib, str(tmp_path / "missing.snap"))
    assert rc == 1 and err == "cannot open the snapshot file"
