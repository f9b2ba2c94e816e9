"""CPU-side checks of the C-ABI boundary: the library builds, loads and
exports every entry point that include/afmib.h declares. No compute calls."""
import ctypes
import os
import shutil
import subprocess

import pytest

from afmibins_gb300 import build, capi


def test_library_exports_declared_symbols():
    lib = capi.load()
    declared = capi.declared_symbols()
    assert len(declared) >= 27
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(capi.declared_symbols()) <= set(capi._SIGS)


def test_error_strings_without_gpu():
    lib = capi.load()
    assert lib.afmib_error_string(capi.AFMIB_OK) == b"ok"
    assert lib.afmib_error_string(capi.AFMIB_ERR_NOCONV) == b"iteration cap reached"
    assert lib.afmib_error_string(99) == b"unknown status"


def test_config_layout_matches_header(tmp_path):
    """The ctypes mirror agrees with the C struct field by field: a C program
    compiled against include/afmib.h prints sizeof and every offsetof."""
    fields = [f[0] for f in capi.Config._fields_]
    src = tmp_path / "layout.c"
    body = "".join(f'    printf("%zu\\n", offsetof(afmib_config, {f}));\n' for f in fields)
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"afmib.h\"\nint main(void) {\n"
                   '    printf("%zu\\n", sizeof(afmib_config));\n' + body + "    return 0;\n}\n")
    exe = tmp_path / "layout"
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    subprocess.run([cc, "-std=c99", "-I", os.path.join(build.ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert out[0] == ctypes.sizeof(capi.Config)
    assert out[1:] == [getattr(capi.Config, f).offset for f in fields]


def test_build_is_in_tree():
    assert capi.library_path().startswith(build.PKG)


@pytest.mark.parametrize("kwargs, words", [
    (dict(nx=8, bc=7), "bc must be"),
    (dict(nx=8, proj_start=3), "proj_start"),
    (dict(nx=8, ny=8, nz=1, bc=capi.BC_CHANNEL), "2D grid"),
    (dict(nx=4096, ny=4096, nz=1), "8192 tiles"),
    (dict(nx=8, dt=0.0), "dt"),
])
def test_create_rejects_bad_configurations_without_gpu(kwargs, words):
    """Configuration checks run before any CUDA call: a bad configuration
    returns AFMIB_ERR_ARG with its reason, and nothing is allocated."""
    nx = kwargs.pop("nx")
    with pytest.raises(capi.AfmibError) as e:
        capi.Solver(nx, **kwargs)
    assert e.value.status == capi.AFMIB_ERR_ARG
    assert words in str(e.value)
