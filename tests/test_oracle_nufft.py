"""Pins the FP64 nufftOp restatement against the reference's own known-answer
tests (operators/@nufftOp/tests.m) and against the direct FP64 NUDFT."""
import numpy as np
import pytest

from oracle.nufft_ref import NufftRef, fftnc, nudft_forward, nudft_adjoint, os_grid_size, kb_table


def _cart_kloc(imN):
    axes = [np.arange(-n / 2, n / 2) / n for n in imN]
    g = np.meshgrid(*axes, indexing="ij")
    return np.stack([a.reshape(-1, order="F") for a in g], axis=1)


def _rand_c(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape) + rng.standard_normal()


@pytest.mark.parametrize("nD", [1, 2, 3])
def test_adjoint_dot(nD):
    # @nufftOp/tests.m:10-37 (os 1.5, kwidth 6, rel < 1e-8)
    rng = np.random.default_rng(nD)
    imN = [32 + 4 * d for d in range(nD)] if nD < 3 else [12, 16, 20]
    kloc = _cart_kloc(imN)
    S = NufftRef(imN, kloc, np.ones(kloc.shape[0]), 1.5, 6)
    x = _rand_c(rng, imN)
    y = _rand_c(rng, (kloc.shape[0],))
    d1 = np.vdot(x.reshape(-1, order="F"), S.H.mtimes(y).reshape(-1, order="F"))
    d2 = np.vdot(S.mtimes(x).reshape(-1, order="F"), y)
    assert abs(d1 - d2) / min(abs(d1), abs(d2)) < 1e-8


@pytest.mark.parametrize("nD", [1, 2])
def test_cartesian_equals_fft(nD):
    # @nufftOp/tests.m:90-101: S*im on a Cartesian kloc, then fftnc, returns im (< 1e-4)
    imN = [32 + 4 * d for d in range(nD)]
    kloc = _cart_kloc(imN)
    rng = np.random.default_rng(3)
    im = rng.uniform(0, 1, imN)
    S = NufftRef(imN, kloc, np.ones(kloc.shape[0]), 1.5, 6)
    k1 = S.mtimes(im).reshape(imN, order="F")
    im1 = fftnc(k1)
    tv = np.sqrt(np.sum(np.abs(im1 - im) ** 2)) / im.size
    assert tv < 1e-4


@pytest.mark.parametrize("nD", [1, 2])
def test_psf(nD):
    # @nufftOp/tests.m:67-88: PSF phase < 1e-6, flatness < 1e-4, scale vs os/kwidth < 1e-3
    imN = [32 + 4 * d for d in range(nD)]
    kloc = _cart_kloc(imN)
    x = np.zeros(imN)
    x[tuple(n // 2 for n in imN)] = 1
    S = NufftRef(imN, kloc, np.ones(kloc.shape[0]), 1.5, 6)
    Sx1 = S.mtimes(x)
    assert np.mean(np.abs(np.angle(Sx1))) < 1e-6
    assert np.std(np.abs(Sx1), ddof=1) / np.mean(np.abs(Sx1)) < 1e-4
    Sx2 = NufftRef(imN, kloc, np.ones(kloc.shape[0]), 1.375, 6).mtimes(x)
    Sx3 = NufftRef(imN, kloc, np.ones(kloc.shape[0]), 1.375, 4).mtimes(x)
    tv = [np.mean(np.abs(Sx1)), np.mean(np.abs(Sx2)), np.mean(np.abs(Sx3))]
    assert np.max(np.abs(np.diff(tv))) < 1e-3


def test_circshift():
    # @nufftOp/tests.m:57-65
    imN = [32, 36]
    kloc = _cart_kloc(imN)
    rng = np.random.default_rng(5)
    y = _rand_c(rng, (kloc.shape[0],))
    a = NufftRef(imN, kloc, np.ones(kloc.shape[0]), 1.5, 6).H.mtimes(y)
    b = NufftRef(imN, kloc + 0.25, np.ones(kloc.shape[0]), 1.5, 6).H.mtimes(y)
    assert abs(np.mean(np.abs(a) - np.abs(b))) < 1e-5


def test_toeplitz():
    # @nufftOp/tests.m:104-124 (2D case): Toeplitz vs an os=2/kw=8 truth, rms < 1e-3
    rng = np.random.default_rng(7)
    imN = [32, 32]
    kloc = rng.uniform(0, 1, (256, 2)) - 0.5
    dcf = rng.uniform(0, 1, 256)
    S = NufftRef(imN, kloc, dcf, 1.5, 6).prepToep()
    x = rng.standard_normal(imN + [2]) + 1j * rng.standard_normal(imN + [2])
    S0 = NufftRef(imN, kloc, dcf, 2, 8)
    y0 = S0.H.mtimes(S0.mtimes(x))
    y1 = S.mtimes(x)
    assert np.sqrt(np.mean(np.abs(y0 - y1) ** 2)) < 1e-3


def test_plan_constants():
    # nufftOp.m:146-165 at kwidth 4, os 2 (Nkern 1522, beta 8.99615) and osN prime factors <= 7
    kern, Nkern, bet = kb_table(4, 2.0)
    assert Nkern == 1522 and abs(bet - 8.996157) < 1e-5 and kern[-1] == 0
    assert os_grid_size([128, 256], 2.0) == [256, 512]
    assert os_grid_size([22], 1.5) == [36]   # 34 = 2*17 -> bumped to 36


def test_against_nudft():
    # Interpolation error of the KB gridding vs the exact FP64 NUDFT (kwidth 4, os 2)
    rng = np.random.default_rng(11)
    imN = [32, 32]
    kloc = rng.uniform(-0.5, 0.5, (500, 2))
    x = rng.standard_normal(imN) + 1j * rng.standard_normal(imN)
    S = NufftRef(imN, kloc, None, 2.0, 4)
    y = S.mtimes(x)
    ye = nudft_forward(imN, kloc, x)
    assert np.linalg.norm(y - ye) / np.linalg.norm(ye) < 2e-3
    yy = rng.standard_normal(500) + 1j * rng.standard_normal(500)
    xa = S.H.mtimes(yy)
    xe = nudft_adjoint(imN, kloc, yy)[..., 0]
    assert np.linalg.norm(xa - xe) / np.linalg.norm(xe) < 2e-3


def test_edge_and_single_samples():
    # samples on the k-space edge (-0.5 and the largest double below 0.5, where the grid index
    # wraps) and a trajectory of one sample keep the gridding error bound against the NUDFT
    rng = np.random.default_rng(13)
    imN = [32, 32]
    kloc = rng.uniform(-0.5, 0.5, (400, 2))
    kloc[:4] = [[-0.5, -0.5], [-0.5, np.nextafter(0.5, 0)], [np.nextafter(0.5, 0), 0.1], [0.0, -0.5]]
    x = rng.standard_normal(imN) + 1j * rng.standard_normal(imN)
    S = NufftRef(imN, kloc, None, 2.0, 4)
    ye = nudft_forward(imN, kloc, x)
    assert np.linalg.norm(S.mtimes(x) - ye) / np.linalg.norm(ye) < 2e-3
    assert np.max(np.abs(S.mtimes(x)[:4] - ye[:4])) / np.max(np.abs(ye[:4])) < 5e-3
    k1 = np.array([[0.123, -0.3]])
    y1 = NufftRef(imN, k1, None, 2.0, 4).mtimes(x)
    assert abs(y1[0] - nudft_forward(imN, k1, x)[0]) / abs(nudft_forward(imN, k1, x)[0]) < 5e-3
