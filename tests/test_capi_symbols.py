"""The C-ABI library builds, loads and exports every entry point that
include/justpic_gb300.h declares (no compute call: this runs without a GPU)."""
import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "justpic_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(jp_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import justpic_gb300 as jp
    from justpic_gb300 import native_build as b
    if b.is_stale():
        if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
            pytest.skip("nvcc not available to build the library")
        jp.build()
    return ctypes.CDLL(b.LIB)


def test_header_declares_the_hot_path():
    syms = declared_symbols()
    for name in ("jp_particles_create", "jp_init_particles", "jp_advection", "jp_move_particles",
                 "jp_inject_particles", "jp_grid2particle", "jp_particle2grid"):
        assert name in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"missing exports: {missing}"


def test_python_binding_covers_the_header():
    from justpic_gb300 import _native
    bound = {name for name, _, _ in _native.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_error_path_without_gpu(lib):
    # argument validation happens before any CUDA call
    lib.jp_particles_create.restype = ctypes.c_int
    lib.jp_last_error.restype = ctypes.c_char_p
    assert lib.jp_particles_create(None, None, 24, 48, 12, 0) == -1
    assert b"null" in lib.jp_last_error()
