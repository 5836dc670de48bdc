"""Pins the FP64 restatements other than nufftOp against the reference's own
known-answer tests: powermethod.m:77-94, @dwtND/tests.m:17-31,
@sampHighOrder/tests.m:10-41 and 265-283, @rcvrOp/tests.m:19-31,
mrSampFunc.m:163-215.  cgne/bfista have no reference tests; they are checked
against their defining properties (exact solve, monotone cost)."""
import numpy as np
import pytest

from oracle.bfista_ref import HaarRef, bfista_ref, powermethod, softthresh
from oracle.nufft_ref import NufftRef, fftnc
from oracle.sense_ref import RcvrRef, cgne_ref, mrsampfunc
from oracle.sho_ref import ShoRef


def crandn(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_powermethod_unit():
    # powermethod.m:77-94 (doAtA = 1): max eig of A'A within 1e-3
    rng = np.random.default_rng(0)
    A = crandn(rng, (8, 5))
    f = lambda x, t: A @ x if t == "notransp" else A.conj().T @ x
    e = powermethod(f, rng.standard_normal(5))
    assert abs(np.max(np.linalg.eigvalsh(A.conj().T @ A)) - e.real) / e.real < 1e-3


@pytest.mark.parametrize("J,shape", [([2, 2], [32, 32]), ([3, 1], [16, 24]), ([2], [40])])
def test_haar_perfect_reconstruction(J, shape):
    # @dwtND/tests.m:17-31: W'W = I for the undecimated transform
    rng = np.random.default_rng(1)
    x = crandn(rng, shape)
    W = HaarRef(J, shape)
    assert np.allclose(W.adjoint(W.forward(x)), x, atol=1e-12)
    b = [crandn(rng, shape) for _ in W.forward(x)]
    d1 = sum(np.vdot(u, v) for u, v in zip(W.forward(x), b))
    d2 = np.vdot(x, W.adjoint(b))
    assert abs(d1 - d2) / abs(d1) < 1e-12


def test_softthresh():
    w = np.array([3 + 4j, 0.1, -2.0, 0j])
    out = softthresh(w, 1.0)
    assert np.allclose(out, [(3 + 4j) * 4 / 5, 0, -1.0, 0])


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_sho_adjoint(nd):
    # @sampHighOrder/tests.m:10-28
    rng = np.random.default_rng(nd)
    imN = [round(64 ** (2 / nd))] * nd
    kN = [round(64 ** (1 / nd))] * nd
    b0 = rng.standard_normal(imN) + rng.uniform()
    t = rng.standard_normal(kN) / np.sqrt(np.prod(kN))
    grid = {k: rng.standard_normal(imN) for k in "xyz"}
    S = ShoRef(b0, t, rng.standard_normal([16] + kN), rng.standard_normal([4] + kN), grid)
    x = crandn(rng, imN + [2])
    y = crandn(rng, kN + [2])
    d1 = np.vdot(x.reshape(-1, order="F"), S.H.mtimes(y).reshape(-1, order="F"))
    d2 = np.vdot(S.mtimes(x).reshape(-1, order="F"), y.reshape(-1, order="F"))
    assert abs(d1 - d2) / min(abs(d1), abs(d2)) < 1e-8


def test_sho_phidiv_is_phase_derivative():
    # setPhiDiv (sampHighOrder.m:590-622, used at 376-380): with phiDiv = the phase coefficients
    # themselves and no B0, S_phiDiv x = d/da [exp(i a kbase).' x / sqrt(V)] at a = 1
    rng = np.random.default_rng(9)
    imN, kN = [12, 10], [200]
    grid = {k: 0.1 * rng.standard_normal(imN) for k in "xyz"}
    spha, conc = rng.standard_normal([16] + kN), rng.standard_normal([4] + kN)
    t = np.linspace(0, 1, kN[0])
    S = ShoRef(None, t, spha, conc, grid)
    x = crandn(rng, imN)
    h = 1e-5
    fd = (ShoRef(None, t, (1 + h) * spha, (1 + h) * conc, grid).mtimes(x)
          - ShoRef(None, t, (1 - h) * spha, (1 - h) * conc, grid).mtimes(x)) / (2 * h)
    got = S.setPhiDiv(spha, conc).mtimes(x)
    assert np.linalg.norm(got - fd) / np.linalg.norm(fd) < 1e-8
    # the adjoint ignores phiDiv (369-372)
    y = crandn(rng, kN)
    assert np.allclose(S.setPhiDiv(spha, conc).H.mtimes(y), S.H.mtimes(y))


def test_sho_fourier():
    # @sampHighOrder/tests.m:265-283: Cartesian linear phase == centered FFT (< 1e-10)
    N = 32
    gx, gy = np.meshgrid(np.arange(-N / 2, N / 2), np.arange(-N / 2, N / 2))
    grid = {"x": gx.astype(float), "y": gy.astype(float), "z": np.zeros((N, N))}
    spha = np.zeros((16, N, N))
    spha[2] = np.pi * 2 / N * np.tile(np.arange(-N / 2, N / 2), N).reshape(N, N, order="F")
    spha[1] = np.pi * 2 / N * np.tile(np.arange(-N / 2, N / 2), (N, 1))
    t = np.arange(N * N, dtype=float).reshape(N, N, order="F")
    im0 = np.random.default_rng(0).uniform(0, 1, (N, N))
    S = ShoRef(np.zeros((N, N)), t, spha, np.zeros((4, N, N)), grid)
    k0 = S.mtimes(im0).reshape(N, N, order="F")
    assert np.sqrt(np.sum((np.abs(k0) - np.abs(fftnc(im0, 2))) ** 2)) / k0.size < 1e-10
    im1 = S.H.mtimes(k0).reshape(N, N, order="F")
    assert np.sqrt(np.sum(np.abs(im1 - im0) ** 2)) / im0.size < 1e-10


def test_rcvr_adjoint():
    # @rcvrOp/tests.m:19-26 (isCalDat = 0)
    rng = np.random.default_rng(2)
    R = RcvrRef(crandn(rng, (32, 32, 4)))
    x, y = crandn(rng, (32, 32)), crandn(rng, (32, 32, 4))
    d1 = np.vdot(x, R.H.mtimes(y))
    d2 = np.vdot(R.mtimes(x), y)
    assert abs(d1 - d2) / min(abs(d1), abs(d2)) < 1e-8


@pytest.mark.parametrize("vec,tik", [(False, False), (True, False), (True, True)])
def test_mrsampfunc_adjoint(vec, tik):
    # mrSampFunc.m:163-215 with a nufftOp sampling operator
    rng = np.random.default_rng(3)
    N, C, M = 32, 2, 400
    S = NufftRef([N, N], rng.uniform(-0.5, 0.5, (M, 2)), None, 2.0, 4)
    R = RcvrRef(crandn(rng, (N, N, C)))
    opt = {"imNFull": [N, N], "daNFull": [M, C]} if vec else {}
    if tik:
        opt["tikReg"] = 0.01
    x = crandn(rng, N * N if vec else (N, N))
    y = crandn(rng, (M * C + (N * N if tik else 0)) if vec else (M, C))
    d1 = np.vdot(x, mrsampfunc(y, "transp", S, R, opt))
    d2 = np.vdot(mrsampfunc(x, "notransp", S, R, opt), y)
    assert abs(d1 - d2) / min(abs(d1), abs(d2)) < 1e-8


def test_cgne_solves_small_system():
    # cgne on a well-conditioned dense system reaches the least-squares solution
    rng = np.random.default_rng(4)
    A = crandn(rng, (40, 12))
    xt = crandn(rng, 12)
    b = A @ xt
    f = lambda x, t: A @ x if t == "notransp" else A.conj().T @ x
    # the explicit-residual restart at nit = 0 (cgne.m:230-246) costs one Krylov step, so run > 12
    x, rs, *_ , status = cgne_ref(f, b, None, 30, {"xChangeThresh": None, "resThresh": None})
    assert np.allclose(x, xt, atol=1e-8)
    assert rs[-1].real < 1e-16 * rs[0].real + 1e-20


def test_bfista_decreases_cost():
    rng = np.random.default_rng(5)
    A = crandn(rng, (256, 64))
    f = lambda x, t: (A @ x.reshape(-1)) if t == "notransp" else (A.conj().T @ x).reshape(8, 8)
    b = A @ crandn(rng, 64)
    x0 = f(b, "transp")          # a zero x0 would make the power method divide by zero, as in the reference
    x, rs, rx, test, me = bfista_ref(f, b, HaarRef([1, 1], [8, 8]), 0.1, x0, 30, {"resThresh": 0})
    cost = rs + rx
    assert cost[-1] < cost[0]


def test_torch_generators_match_numpy():
    torch = pytest.importorskip("torch")
    from matmri_gb300 import synth
    img = synth.ellipse_phantom(48, 10, 7, complex_phase=True)
    it = synth.ellipse_phantom_torch(48, 10, 7, complex_phase=True, device="cpu").numpy()
    assert np.abs(it - img).max() < 1e-6
    m = synth.coil_maps(40, 6, 3, randomize=True)
    mt = synth.coil_maps_torch(40, 6, 3, randomize=True, device="cpu")
    assert mt.shape == (40, 40, 6) and mt.stride() == (1, 40, 1600)
    assert np.abs(mt.numpy() - m).max() < 1e-6


def test_dense_normal_matrix_equals_operator_normal():
    # mrSampFuncMat.m:22-47 with a full mask: AtA x == R'S'SR x and Aty == R'S'y
    from oracle.densemat_ref import mrsampfuncmat_ref
    from oracle.sense_ref import RcvrRef, mrsampfunc
    rng = np.random.default_rng(4)
    N, M, C = 10, 150, 3
    c = (np.arange(N) - N / 2) * 0.02
    X, Y = np.meshgrid(c, c, indexing="ij")
    grid = {"x": X, "y": Y, "z": np.zeros_like(X)}
    spha = np.zeros((16, M))
    spha[1:3] = rng.uniform(-150, 150, (2, M))
    spha[4] = rng.uniform(-300, 300, M)
    t = np.linspace(0, 0.01, M)
    b0 = rng.uniform(-50, 50, (N, N))
    maps = crandn(rng, (N, N, C))
    y = crandn(rng, (M, C))
    AtA, Aty = mrsampfuncmat_ref(y, maps, b0, t, spha, np.zeros((4, M)), grid)
    S, R = ShoRef(b0, t, spha, np.zeros((4, M)), grid), RcvrRef(maps)
    x = crandn(rng, (N, N))
    ref = mrsampfunc(mrsampfunc(x, "notransp", S, R), "transp", S, R).reshape(-1, order="F")
    assert np.linalg.norm(AtA @ x.reshape(-1, order="F") - ref) < 1e-10 * np.linalg.norm(ref)
    assert np.allclose(Aty, mrsampfunc(y, "transp", S, R).reshape(-1, order="F"), atol=1e-12)
    assert np.allclose(AtA, AtA.conj().T, atol=1e-12)
