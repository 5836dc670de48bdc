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


def test_nufft_plan_validation_without_gpu(lib):
    # nufftOp arguments are validated before any CUDA call: odd image extents (the reference's
    # phase ramp is then a half-cell shift), odd or too wide kernels, no samples, NaN trajectories
    from matmri_gb300 import _lib
    import numpy as np

    def create(imN, kloc, kwidth=4, os_=2.0):
        kl = np.asfortranarray(kloc, dtype=np.float64)
        d = _lib.NufftDesc()
        d.ndim = len(imN)
        for i, n in enumerate(imN):
            d.imN[i] = n
        d.nsamp = kl.shape[0]
        d.kloc = kl.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.dcf = None
        d.os = os_
        d.kwidth = kwidth
        out = ctypes.c_void_p()
        code = lib.mmr_nufft_create(ctypes.byref(d), ctypes.byref(out))
        buf = ctypes.create_string_buffer(512)
        lib.mmr_last_error(buf, 512)
        return code, buf.value.decode()

    k = np.random.default_rng(0).uniform(-0.5, 0.5, (16, 2))
    code, msg = create([33, 32], k)
    assert code == 1 and "even" in msg
    code, msg = create([32, 32], k, kwidth=5)
    assert code == 1 and "kwidth" in msg
    code, msg = create([32, 32], k, kwidth=10)
    assert code == 1 and "kwidth" in msg
    code, msg = create([32, 32], k[:0])
    assert code == 1 and "sample" in msg
    bad = k.copy()
    bad[3, 1] = np.nan
    code, msg = create([32, 32], bad)
    assert code == 1 and "NaN" in msg
