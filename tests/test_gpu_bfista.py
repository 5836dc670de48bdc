"""powermethod, the undecimated Haar dwtND and bfista on the GPU against the
FP64 restatement (iterativeSolvers/powermethod.m, operators/@dwtND,
iterativeSolvers/bfista.m)."""
import numpy as np
import pytest

from gpu_util import crandn, rel
from oracle.bfista_ref import HaarRef, bfista_ref, powermethod as pm_ref
from oracle.nufft_ref import NufftRef
from oracle.sense_ref import RcvrRef, mrsampfunc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mm():
    import matmri_gb300 as m
    return m


@pytest.mark.parametrize("J,shape", [([2, 2], [64, 48]), ([3, 1], [32, 32]), ([1, 0], [16, 20]), ([2], [64])])
def test_haar_bands_and_inverse(mm, J, shape):
    rng = np.random.default_rng(len(shape) * 7 + J[0])
    x = crandn(rng, shape)
    Wg = mm.dwtND(J, shape)
    Wr = HaarRef(J, shape)
    bands = Wg * x
    ref = Wr.forward(x)
    assert len(bands) == len(ref)
    for a, b in zip(bands, ref):
        assert rel(a, b) < 1e-6
    # W'W = I for the undecimated transform (@dwtND/tests.m:17-31)
    assert rel(Wg.H * bands, x) < 1e-6
    # adjoint identity
    wb = [crandn(rng, shape) for _ in bands]
    d1 = sum(np.vdot(b, w) for b, w in zip(bands, wb))
    d2 = np.vdot(x, Wg.H * wb)
    assert abs(d1 - d2) / abs(d1) < 1e-5


def _sense(mm, seed=0, N=64, C=4, M=3000):
    from matmri_gb300 import synth
    rng = np.random.default_rng(seed)
    kloc = synth.spiral(N, 4, M // 4, 2.0)
    maps = synth.coil_maps(N, C, seed)
    S = mm.nufftOp([N, N], kloc, None, 1, 2.0, 4)
    R = mm.rcvrOp(maps, 0)
    Sr, Rr = NufftRef([N, N], kloc, None, 2.0, 4), RcvrRef(maps)
    img = synth.ellipse_phantom(N, 10, seed, complex_phase=True)
    data = synth.add_noise(mrsampfunc(img, "notransp", Sr, Rr), 20.0, seed + 5)
    return mm.mrSampOp(S, R), (lambda v, t: mrsampfunc(v, t, Sr, Rr)), data, img


def test_powermethod(mm):
    A, Aref, data, img = _sense(mm, seed=1)
    x0 = np.random.default_rng(3).standard_normal((64, 64)).astype(complex)
    e = mm.powermethod(A, x0)
    er = pm_ref(Aref, x0)
    assert abs(e - er) / abs(er) < 1e-4


@pytest.mark.parametrize("lam_kind", ["scalar", "per_band"])
def test_bfista_vs_oracle(mm, lam_kind):
    A, Aref, data, img = _sense(mm, seed=2)
    J = [2, 2]
    W = mm.dwtND(J, [64, 64])
    nb = W.nbands
    lam = 2e-3 if lam_kind == "scalar" else [0.0] + [2e-3] * (nb - 1)     # demos/demo_wavelet.m:101-102
    x0 = Aref(data, "transp")
    maxEig = float(abs(pm_ref(Aref, x0)))
    opt = {"maxEig": maxEig, "resThresh": 1e-9}
    x, rs, rx, test, me = mm.bfista(A, data, W, lam, x0, 15, opt)
    xr, rsr, rxr, testr, mer = bfista_ref(Aref, data, HaarRef(J, [64, 64]), lam, x0, 15, opt)
    assert len(rs) == len(rsr) == 15
    assert rel(x, xr) < 1e-4
    assert np.allclose(rs, rsr, rtol=1e-3)
    assert np.allclose(rx, rxr, rtol=1e-3)


def test_bfista_stops_on_resthresh(mm):
    A, Aref, data, img = _sense(mm, seed=4)
    W = mm.dwtND([1, 1], [64, 64])
    x0 = Aref(data, "transp")
    opt = {"resThresh": 5e-2}                     # maxEig from the power method (bfista.m:81-89)
    x, rs, rx, test, me = mm.bfista(A, data, W, 1e-3, x0, 50, opt)
    xr, rsr, rxr, testr, mer = bfista_ref(Aref, data, HaarRef([1, 1], [64, 64]), 1e-3, x0, 50, opt)
    assert abs(me - abs(mer)) / abs(mer) < 1e-3
    assert len(rs) == len(rsr) < 50
