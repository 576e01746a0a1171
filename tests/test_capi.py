"""CPU checks of the product library: it builds, loads, and exports every
entry point include/rive_cuda.h declares (no GPU calls)."""
import ctypes
import os
import subprocess

from conftest import REPO, load_package

pkg = load_package()
from rive_runtime_gb300 import build, rive_cuda  # noqa: E402


def test_library_builds_and_exports_header_symbols():
    lib_path = build.build()
    assert os.path.exists(lib_path)
    lib = ctypes.CDLL(lib_path)
    names = rive_cuda.exported_functions()
    assert "rive_cuda_flush" in names and "rive_cuda_context_create" in names
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True,
                         text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_binding_declares_every_header_function():
    rive_cuda.load()
    for n in rive_cuda.exported_functions():
        fn = getattr(rive_cuda.load(), n)
        assert fn.argtypes is not None, f"{n} has no ctypes signature"


def test_null_arguments_are_rejected_without_a_gpu_call():
    lib = rive_cuda.load()
    assert lib.rive_cuda_context_create(0, None) == 1  # RIVE_CUDA_ERR_INVALID_ARGUMENT
    assert lib.rive_cuda_last_error(None, None, 0) == 1
    assert lib.rive_cuda_map_buffer(None, 0, 16) is None


def test_feather_table_is_the_oracles():
    """The library's feather table (host code, no GPU needed) equals the
    oracle's, which is pinned to the reference's shipped table."""
    from rive_runtime_gb300 import rive_cuda
    import oracle
    assert (rive_cuda.feather_table() == oracle.feather_table()).all()


def test_inverse_feather_table_is_the_oracles():
    """The library's inverse feather table (host code, no GPU needed) equals the
    oracle's, which equals the reference's shipped table."""
    from rive_runtime_gb300 import rive_cuda
    import oracle
    assert (rive_cuda.inverse_feather_table() == oracle.inverse_feather_table()).all()
