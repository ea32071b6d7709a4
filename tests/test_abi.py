"""C-ABI checks that need no GPU: the library builds, loads, exports every
entry point include/gbr.h declares, and rejects bad arguments with a status
code instead of exiting or throwing."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbr.h")


def declared_symbols():
    text = open(HEADER).read()
    decl = r"^(?:gbr_status|const char \*|uint32_t|void)\s*\*?\s*(gbr_[a-z_]+)\s*\("
    return sorted(set(re.findall(decl, text, flags=re.M)))


def test_header_declares_the_binding_surface(gbr_lib):
    assert sorted(gbr_lib.EXPORTED) == declared_symbols()


def test_library_exports_every_declared_symbol(gbr_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", gbr_lib.library_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (gbr_[a-z_]+)\b", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    L = gbr_lib.lib()
    for s in declared_symbols():
        assert getattr(L, s) is not None


def test_version_and_error_string(gbr_lib):
    L = gbr_lib.lib()
    assert L.gbr_version() == 0x000100
    assert isinstance(L.gbr_last_error_string(), bytes)


def test_invalid_arguments_return_status(gbr_lib):
    L = gbr_lib.lib()
    assert L.gbr_create(640, 480, None) == 1
    h = C.c_void_p()
    assert L.gbr_create(0, 480, C.byref(h)) == 1
    assert b"resolution" in L.gbr_last_error_string()
    assert L.gbr_create(9000, 480, C.byref(h)) == 1
    assert L.gbr_setup_bins(None, 1, 1, 16, 16, 0) == 1
    assert L.gbr_render(None, None, 0, 0, 0, None) == 1
    assert L.gbr_readback(None, None, None, None) == 1
    assert L.gbr_destroy(None) == 0


def test_public_header_compiles_as_c():
    src = '#include "gbr.h"\nint main(void){ gbr_stats s; (void)s; return (int)GBR_OK; }\n'
    p = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-x", "c", "-",
                        "-fsyntax-only"], input=src, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


def test_create_without_gpu_fails_cleanly(gbr_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = gbr_lib.lib()
    h = C.c_void_p()
    st = L.gbr_create(64, 64, C.byref(h))
    assert st == 2 and not h.value
    assert len(L.gbr_last_error_string()) > 0
