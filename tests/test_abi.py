"""The C-ABI library builds, loads, and exports every entry point that include/*.h declares.

No compute call is made here (no GPU in the CPU suite)."""
import pathlib
import re

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"\b(plgpu_\w+)\s*\(", text))
    return names


def test_header_declares_the_abi():
    names = declared_functions()
    for n in ("plgpu_fem3d_create", "plgpu_fem3d_compute", "plgpu_fem3d_get_temperature", "plgpu_fem3d_destroy"):
        assert n in names


def test_library_loads_and_exports_every_declared_symbol():
    from plask_gb300 import _native

    lib = _native.load()
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers the whole header
    assert declared_functions() <= set(_native.SIGNATURES)


def test_library_is_in_tree_and_built_for_sm103a():
    from plask_gb300 import _native, build

    assert _native.library_path().parent == ROOT / "plask_gb300" / "lib"
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)


def test_creation_error_without_gpu_is_reported_not_raised_in_c():
    """create() on a machine without a GPU returns an error code with a message (no crash)."""
    import numpy as np

    from plask_gb300 import _native

    try:
        import torch

        if torch.cuda.is_available():
            return
    except Exception:
        pass
    try:
        _native.Fem3D((np.linspace(0, 1, 3),) * 3)
    except _native.NativeError as e:
        assert e.code != 0
    else:
        raise AssertionError("expected a CUDA error without a GPU")


def test_headers_are_plain_c_and_the_library_links_from_c(tmp_path):
    """A C99 program that includes every header and takes the address of every declared
    entry point compiles warning-free and links against the library: the boundary a
    cgo, JNI or ctypes binding sees, with no C++ type in it."""
    import shutil
    import subprocess

    import pytest

    from plask_gb300 import _native

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    lib = _native.load() and _native.library_path()
    names = sorted(declared_functions())
    headers = sorted(p.name for p in (ROOT / "include").glob("*.h"))
    src = ["#include <stdio.h>"] + [f'#include "{h}"' for h in headers]
    src += ["typedef void (*entry_point)(void);", "static const entry_point entry_points[] = {"]
    src += [f"    (entry_point){n}," for n in names]
    src += ["};", "int main(void) {",
            '    printf("%u\\n", (unsigned)(sizeof entry_points / sizeof entry_points[0]));', "    return 0;", "}"]
    c = tmp_path / "abi.c"
    c.write_text("\n".join(src) + "\n")
    exe = tmp_path / "abi"
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(c), "-L",
           str(lib.parent), "-lplgpu_fem3d", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert int(out.stdout.strip()) == len(names)
