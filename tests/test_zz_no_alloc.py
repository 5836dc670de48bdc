"""The allocation-free nufftOp adjoint (mmr_nufft_adjoint_noalloc).

Callers that cannot allocate device memory while they apply the operator —
a MEX or plug-in held to a fixed device budget by its host application, a
real-time loop that must not call cudaMalloc — use this entry point; its
grid scratch is a fixed array in the library's device image.  The
test calls it through the C ABI twice in a row (the array keeps the first
call's contents) and compares each result with the regular adjoint
mmr_nufft_apply(adjoint = 1) at the tolerance of the other GPU tests.  This
file sorts last so that a run stopping at the first failure has already run
every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("imN,M,nb,os_,kw,dcf", [([128, 128], 6000, 3, 2.0, 4, True),
                                                 ([64, 48], 2000, 2, 1.5, 6, False),
                                                 ([96], 400, 4, 2.0, 4, True),
                                                 ([12, 16, 10], 900, 2, 2.0, 4, True)])
def test_noalloc_adjoint_matches_apply(imN, M, nb, os_, kw, dcf):
    torch = pytest.importorskip("torch")
    import matmri_gb300 as mm
    from matmri_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(M)
    kloc = rng.uniform(-0.5, 0.5, (M, len(imN)))
    N = mm.nufftOp(imN, kloc, rng.uniform(0.2, 1.0, M) if dcf else None, 1, os_, kw)
    for call in range(2):
        y = (rng.standard_normal((M, nb)) + 1j * rng.standard_normal((M, nb))).astype(np.complex64)
        yd = torch.from_numpy(np.asfortranarray(y).T.copy()).cuda()          # column-major [M, nb]
        xa = torch.empty(nb * int(np.prod(imN)), dtype=torch.complex64, device="cuda")
        xb = torch.empty_like(xa)
        _lib.check(lib.mmr_nufft_apply(N.handle, 1, yd.data_ptr(), xa.data_ptr(), nb, None))
        _lib.check(lib.mmr_nufft_adjoint_noalloc(N.handle, yd.data_ptr(), xb.data_ptr(), nb, None))
        torch.cuda.synchronize()
        assert _rel(xb.cpu().numpy(), xa.cpu().numpy()) < TOL, f"call {call}"


def test_noalloc_rejects_oversize_and_host_pointers():
    pytest.importorskip("torch")
    import matmri_gb300 as mm
    from matmri_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(1)
    N = mm.nufftOp([512, 512], rng.uniform(-0.5, 0.5, (1000, 2)), None, 1, 2.0, 4)   # 1024^2 grid > 1 Mi values
    y = np.zeros((1000, 1), np.complex64)
    x = np.zeros((512, 512), np.complex64)
    assert lib.mmr_nufft_adjoint_noalloc(N.handle, y.ctypes.data, x.ctypes.data, 1, None) == 1
    import torch
    yd = torch.zeros(1000, dtype=torch.complex64, device="cuda")
    xd = torch.zeros(512 * 512, dtype=torch.complex64, device="cuda")
    assert lib.mmr_nufft_adjoint_noalloc(N.handle, yd.data_ptr(), xd.data_ptr(), 1, None) == 1
    buf = C.create_string_buffer(512)
    lib.mmr_last_error(buf, 512)
    assert b"scratch" in buf.value
    # a batch count so large that nbatch * (scratch per column) would wrap a 64-bit size is rejected
    # before anything is launched
    Ns = mm.nufftOp([16, 16], rng.uniform(-0.5, 0.5, (100, 2)), None, 1, 2.0, 4)
    ys = torch.zeros(100, dtype=torch.complex64, device="cuda")
    xs = torch.zeros(256, dtype=torch.complex64, device="cuda")
    for nb in (2 ** 62, 2 ** 63 - 1, 1 << 20):
        assert lib.mmr_nufft_adjoint_noalloc(Ns.handle, ys.data_ptr(), xs.data_ptr(), nb, None) == 1
