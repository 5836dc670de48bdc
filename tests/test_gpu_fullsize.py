"""The CG-SENSE path at the headline size (256 x 256, 32 coils, 4 x 4096 spiral at R = 4,
kwidth 4, os 2) with the launch shapes the autotuner picks for it and with the defaults:
parity with the FP64 restatement (operators/mrSampFunc.m, @nufftOp, @rcvrOp,
iterativeSolvers/cgne.m) and the size-independent identities of the operators."""
import numpy as np
import pytest

from gpu_util import crandn, rel
from oracle.nufft_ref import NufftRef
from oracle.sense_ref import RcvrRef, cgne_ref, mrsampfunc

pytestmark = pytest.mark.gpu
TOL = 1e-5

# (coil_chunk, tile, coil_group, item, fft_lines, normal_mode): the autotuner's choice on a
# GB300 for this workload, the same with 16 coils per pass, and the stencil gridding form
TUNINGS = [(32, 16, 4, 256, 4, 1), (16, 32, 2, 128, 4, 1), (32, 32, 2, 256, 4, 2)]


@pytest.fixture(scope="module")
def case():
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    c = synth.sense_case(256, 32, 4, 4096, 4.0, seed=2000)
    Sr = NufftRef([256, 256], c["kloc"], None, 2.0, 4)
    Rr = RcvrRef(c["maps"])
    return mm, c, Sr, Rr


def _op(mm, c, tuning):
    A = mm.mrSampOp(mm.nufftOp([256, 256], c["kloc"], None, 1, 2.0, 4), mm.rcvrOp(c["maps"], 0))
    if tuning is not None:
        A.set_tuning(*tuning)
        assert A.get_tuning() == tuning
    return A


@pytest.mark.parametrize("tuning", TUNINGS + [None])
def test_normal_operator_matches_fp64(case, tuning):
    mm, c, Sr, Rr = case
    A = _op(mm, c, tuning)
    x = crandn(np.random.default_rng(1), (256, 256))
    ref = mrsampfunc(mrsampfunc(x, "notransp", Sr, Rr), "transp", Sr, Rr)
    assert rel(A.normal(x), ref) < TOL


def test_forward_adjoint_match_fp64_and_identities(case):
    mm, c, Sr, Rr = case
    A = _op(mm, c, TUNINGS[0])
    rng = np.random.default_rng(2)
    x = crandn(rng, (256, 256))
    y = crandn(rng, (c["kloc"].shape[0], 32))
    Ax = A(x, "notransp")
    Ahy = A(y, "transp")
    assert rel(Ax, mrsampfunc(x, "notransp", Sr, Rr)) < TOL
    assert rel(Ahy, mrsampfunc(y, "transp", Sr, Rr)) < TOL
    # adjoint identity <A x, y> = <x, A' y>
    lhs = np.vdot(Ax.reshape(-1), y.reshape(-1))
    rhs = np.vdot(x.reshape(-1), Ahy.reshape(-1))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
    # the fused normal operator is Hermitian, positive, linear, and equals A'(A x)
    z = crandn(rng, (256, 256))
    Nx, Nz = A.normal(x), A.normal(z)
    assert abs(np.vdot(z, Nx) - np.vdot(Nz, x)) / abs(np.vdot(z, Nx)) < 1e-5
    q = np.vdot(x, Nx)
    assert q.real > 0 and abs(q.imag) / q.real < 1e-5
    assert rel(A.normal(2.0 * x - 0.5j * z), 2.0 * Nx - 0.5j * Nz) < 1e-5
    assert rel(Nx, A(Ax, "transp")) < TOL


@pytest.mark.parametrize("nit,tol", [(3, 1e-4), (10, 1e-3)])
def test_cgne_matches_fp64(case, nit, tol):
    # The operators agree with FP64 to 1e-5 per application (above); CG amplifies their FP32
    # rounding with the iterations at this size and conditioning (about 3.6e-4 after 10), so the
    # iterate's tolerance grows with nit.  The residual vector is complex64: its recursively
    # updated norm carries errors of order 1e-7 |r0|, which matter once |r| falls below 1e-4 |r0|,
    # so residual norms must agree to 1e-3 relative or to 1e-6 |r0|; |x|^2 to twice the iterate's
    # tolerance.
    mm, c, Sr, Rr = case
    from matmri_gb300 import synth
    A = _op(mm, c, TUNINGS[0])
    data = synth.add_noise(mrsampfunc(c["img"], "notransp", Sr, Rr), 30.0, 2001)
    opt = {"xChangeThresh": None, "resThresh": None}
    x, rs, _, xn, _, _, status = mm.cgne(A, data, None, nit, opt)
    Aref = lambda v, t: mrsampfunc(v, t, Sr, Rr)
    xr, rsr, _, xnr, _, _, statr = cgne_ref(Aref, data, None, nit, opt)
    assert status == statr == 0 and len(rs) == len(rsr) == nit + 1
    assert rel(x, xr) < tol
    r, rr = np.sqrt(np.asarray(rs)), np.sqrt(rsr.real)
    assert np.all(np.abs(r - rr) <= 1e-3 * rr + 1e-6 * rr[0])
    assert np.allclose(xn, xnr.real, rtol=2 * tol)
