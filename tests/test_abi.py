"""CPU checks of the C ABI: the library builds, loads, and exports every
symbol include/matmri_gb300.h declares (no compute call needs a GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "matmri_gb300.h")


def declared():
    txt = open(HDR).read()
    return sorted(set(re.findall(r"^MMR_API\s+int\s+(mmr_\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from matmri_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared()
    assert len(names) >= 25
    for must in ("mmr_nufft_create", "mmr_nufft_apply", "mmr_sense_normal", "mmr_cgne_solve", "mmr_sho_apply"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared():
        assert hasattr(lib, name), name


def test_abi_version_and_error_buffer(lib):
    assert lib.mmr_abi_version() == 1
    buf = ctypes.create_string_buffer(16)
    assert lib.mmr_last_error(buf, 16) == 0
    assert lib.mmr_last_error(None, 0) != 0


def test_binding_signatures_cover_header():
    from matmri_gb300 import _lib
    assert set(declared()) <= set(_lib.SIGNATURES)


def test_null_arguments_are_rejected_without_gpu(lib):
    # argument validation happens before any CUDA call
    out = ctypes.c_void_p()
    assert lib.mmr_nufft_create(None, ctypes.byref(out)) == 1
    assert lib.mmr_sense_create(None, ctypes.byref(out)) == 1
