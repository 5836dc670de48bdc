"""nufftOp on the GPU against the FP64 restatement (per-application rel-L2
<= 1e-5) and the reference's own known-answer identities
(operators/@nufftOp/tests.m)."""
import numpy as np
import pytest

from gpu_util import cart_kloc, crandn, rel
from oracle.nufft_ref import NufftRef, fftnc, nudft_forward

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def mm():
    import matmri_gb300 as m
    return m


CASES = [
    # imN, M, os, kwidth
    ([64], 300, 2.0, 4),
    ([64, 48], 2000, 2.0, 4),
    ([32, 36], 900, 1.5, 6),
    ([128, 128], 6000, 2.0, 4),
    ([48, 48], 1500, 1.375, 4),
    ([16, 20, 12], 1200, 2.0, 4),
    ([64, 64], 3000, 2.0, 8),
    ([64, 64], 3000, 2.0, 2),
]


@pytest.mark.parametrize("imN,M,os_,kw", CASES)
def test_forward_adjoint_vs_oracle(mm, imN, M, os_, kw):
    rng = np.random.default_rng(len(imN) * 100 + M)
    kloc = rng.uniform(-0.5, 0.5, (M, len(imN)))
    dcf = rng.uniform(0.2, 1.0, M)
    ref = NufftRef(imN, kloc, dcf, os_, kw)
    N = mm.nufftOp(imN, kloc, dcf, 1, os_, kw)
    assert N.osN == ref.osN
    x = crandn(rng, imN + [3])
    y = crandn(rng, (M, 3))
    assert rel(N * x, ref.mtimes(x)) < TOL
    assert rel(N.H * y, ref.H.mtimes(y)) < TOL


def test_dcf_setter_and_clear(mm):
    rng = np.random.default_rng(3)
    imN, M = [64, 64], 2500
    kloc = rng.uniform(-0.5, 0.5, (M, 2))
    N = mm.nufftOp(imN, kloc, None, 1, 2.0, 4)
    dcf = rng.uniform(0, 1, M)
    N.dcf = dcf
    y = crandn(rng, M)
    assert rel(N.H * y, NufftRef(imN, kloc, dcf, 2.0, 4).H.mtimes(y)) < TOL
    N.dcf = None
    assert rel(N.H * y, NufftRef(imN, kloc, None, 2.0, 4).H.mtimes(y)) < TOL


@pytest.mark.parametrize("nD", [1, 2, 3])
def test_adjoint_dot(mm, nD):
    # @nufftOp/tests.m:30-37 (rel 1e-8 there in FP64; complex64 here: 1e-5)
    imN = [32 + 4 * d for d in range(nD)] if nD < 3 else [12, 16, 20]
    kloc = cart_kloc(imN)
    rng = np.random.default_rng(nD)
    S = mm.nufftOp(imN, kloc, np.ones(kloc.shape[0]), 1, 1.5, 6)
    x = crandn(rng, imN)
    y = crandn(rng, kloc.shape[0])
    d1 = np.vdot(x.reshape(-1, order="F"), (S.H * y).reshape(-1, order="F"))
    d2 = np.vdot((S * x).reshape(-1, order="F"), y)
    assert abs(d1 - d2) / min(abs(d1), abs(d2)) < 1e-5


@pytest.mark.parametrize("nD", [1, 2])
def test_cartesian_equals_fft(mm, nD):
    # @nufftOp/tests.m:90-101
    imN = [32 + 4 * d for d in range(nD)]
    kloc = cart_kloc(imN)
    im = np.random.default_rng(9).uniform(0, 1, imN)
    S = mm.nufftOp(imN, kloc, np.ones(kloc.shape[0]), 1, 1.5, 6)
    k1 = np.reshape(S * im, imN, order="F")
    im1 = fftnc(k1)
    assert np.sqrt(np.sum(np.abs(im1 - im) ** 2)) / im.size < 1e-4


def test_psf(mm):
    # @nufftOp/tests.m:67-81 (phase < 1e-6 there in FP64; complex64 here)
    imN = [32, 36]
    kloc = cart_kloc(imN)
    x = np.zeros(imN)
    x[16, 18] = 1
    S = mm.nufftOp(imN, kloc, np.ones(kloc.shape[0]), 1, 1.5, 6)
    y = S * x
    assert np.mean(np.abs(np.angle(y))) < 1e-5
    assert np.std(np.abs(y), ddof=1) / np.mean(np.abs(y)) < 1e-4


def test_circshift(mm):
    # @nufftOp/tests.m:57-65: kloc outside [-0.5, 0.5) wraps
    imN = [32, 36]
    kloc = cart_kloc(imN)
    y = crandn(np.random.default_rng(5), kloc.shape[0])
    a = mm.nufftOp(imN, kloc, np.ones(kloc.shape[0]), 1, 1.5, 6).H * y
    b = mm.nufftOp(imN, kloc + 0.25, np.ones(kloc.shape[0]), 1, 1.5, 6).H * y
    assert abs(np.mean(np.abs(a) - np.abs(b))) < 1e-5


def test_binned_path_tiles_agree(mm):
    # every tile size of the binned 2D kernels gives the same result as the oracle
    rng = np.random.default_rng(17)
    imN, M = [128, 128], 8000
    kloc = rng.uniform(-0.5, 0.5, (M, 2))
    ref = NufftRef(imN, kloc, None, 2.0, 4)
    x = crandn(rng, imN + [4])
    y = crandn(rng, (M, 4))
    R = mm.rcvrOp(np.ones(imN + [1], dtype=np.complex64), 0)
    for tile, cgrp, item in ((8, 1, 8), (16, 2, 16), (32, 4, 64), (64, 8, 256), (32, 8, 100000)):
        N = mm.nufftOp(imN, kloc, None, 1, 2.0, 4)
        op = mm.mrSampOp(N, None)
        op.set_tuning(0, tile, cgrp, item)
        assert op.get_tuning()[1:4] == (tile, cgrp, item)
        assert rel(N * x, ref.mtimes(x)) < TOL
        assert rel(N.H * y, ref.H.mtimes(y)) < TOL


def test_error_vs_nudft(mm):
    # kwidth 4 / os 2 gridding error against the exact FP64 NUDFT (stated in the design notes)
    rng = np.random.default_rng(21)
    imN, M = [64, 64], 3000
    kloc = rng.uniform(-0.5, 0.5, (M, 2))
    x = crandn(rng, imN)
    N = mm.nufftOp(imN, kloc, None, 1, 2.0, 4)
    e = rel(N * x, nudft_forward(imN, kloc, x))
    assert e < 2e-3


def test_toeplitz(mm):
    # @nufftOp/tests.m:104-124 (2D): Toeplitz normal op vs an os 2 / kwidth 8 truth
    rng = np.random.default_rng(7)
    imN = [64, 64]
    kloc = rng.uniform(0, 1, (1024, 2)) - 0.5
    dcf = rng.uniform(0, 1, 1024)
    S = mm.nufftOp(imN, kloc, dcf, 1, 1.5, 6).prepToep()
    x = crandn(rng, imN + [2])
    ref = NufftRef(imN, kloc, dcf, 1.5, 6).prepToep()
    y1 = S * x
    assert rel(y1, ref.mtimes(x)) < 1e-5
    S0 = NufftRef(imN, kloc, dcf, 2, 8)
    y0 = S0.H.mtimes(S0.mtimes(x))
    assert np.sqrt(np.mean(np.abs(y0 - y1) ** 2)) < 1e-3


def test_torch_device_tensors(mm):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    imN, M = [64, 64], 2000
    kloc = rng.uniform(-0.5, 0.5, (M, 2))
    N = mm.nufftOp(imN, kloc, None, 1, 2.0, 4)
    x = crandn(rng, imN).astype(np.complex64)
    xt = torch.from_numpy(x).cuda()
    yt = N * xt
    assert yt.is_cuda and yt.dtype == torch.complex64
    assert rel(yt.cpu().numpy(), N * x) < 1e-6
