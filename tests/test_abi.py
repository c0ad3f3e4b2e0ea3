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
