"""The C-ABI library loads and exports every entry point include/uwgpu.h declares (no GPU calls)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "uwgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(uwgpu_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("uwgpu_create", "uwgpu_bin_and_map", "uwgpu_assemble", "uwgpu_solve_bsscr", "uwgpu_operator_apply"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from earthbyte_underworld_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.uwgpu_abi_version() == 2


def test_create_without_device_fails_cleanly():
    """On a machine without a usable GPU, uwgpu_create reports an error instead of falling back."""
    import pytest
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from earthbyte_underworld_gb300 import uwgpu as U
    with pytest.raises(U.UwgpuError):
        U.Context(0)


def test_c_host_program_builds_against_the_abi():
    """The C host side (the reference's own language) compiles and links against libuwgpu.so."""
    from earthbyte_underworld_gb300 import build
    build.build()
    assert os.path.exists(build.build_host())
