"""sampHighOrder on the GPU against the FP64 restatement and the reference's
known-answer tests (operators/@sampHighOrder/tests.m)."""
import numpy as np
import pytest

from gpu_util import crandn, rel
from oracle.nufft_ref import fftnc
from oracle.sho_ref import ShoRef

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mm():
    import matmri_gb300 as m
    return m


def _rand_case(rng, imN, kN):
    b0 = rng.standard_normal(imN) + rng.uniform()
    t = rng.standard_normal(kN) / np.sqrt(np.prod(kN))
    spha = rng.standard_normal([16] + list(kN))
    conc = rng.standard_normal([4] + list(kN))
    grid = {k: rng.standard_normal(imN) for k in "xyz"}
    return b0, t, spha, conc, grid


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_random_vs_oracle_and_adjoint(mm, nd):
    # @sampHighOrder/tests.m:10-28 shapes (N0 = 64)
    rng = np.random.default_rng(nd)
    N0 = 64
    imN = [round(N0 ** (2 / nd))] * nd
    kN = [round(N0 ** (1 / nd))] * nd
    b0, t, spha, conc, grid = _rand_case(rng, imN, kN)
    S = mm.sampHighOrder(b0, t, spha, conc, grid, None, 1, 0, 0)
    Sr = ShoRef(b0, t, spha, conc, grid)
    x = crandn(rng, imN + [2])
    y = crandn(rng, kN + [2])
    assert rel(S * x, Sr.mtimes(x)) < 1e-5
    assert rel(S.H * y, Sr.H.mtimes(y)) < 1e-5
    d1 = np.vdot(x.reshape(-1, order="F"), (S.H * y).reshape(-1, order="F"))
    d2 = np.vdot((S * x).reshape(-1, order="F"), y.reshape(-1, order="F"))
    assert abs(d1 - d2) / min(abs(d1), abs(d2)) < 1e-5


def test_segmented_approaches_equal(mm):
    # @sampHighOrder/tests.m:30-41: approaches 2 and 3 equal the direct one
    rng = np.random.default_rng(4)
    b0, t, spha, conc, grid = _rand_case(rng, [16, 16], [64])
    x = crandn(rng, (16, 16, 2))
    ys = [mm.sampHighOrder(b0, t, spha, conc, grid, None, 1, 0, a, {"segmentedNdiv": 2}) * x for a in (0, 2, 3)]
    assert rel(ys[1], ys[0]) < 1e-6 and rel(ys[2], ys[0]) < 1e-6


def test_fourier_equivalence(mm):
    # @sampHighOrder/tests.m:265-283 (phase = Cartesian linear ramp -> centered FFT)
    N = 64
    gx, gy = np.meshgrid(np.arange(-N / 2, N / 2), np.arange(-N / 2, N / 2))
    grid = {"x": gx.astype(float), "y": gy.astype(float), "z": np.zeros((N, N))}
    spha = np.zeros((16, N, N))
    conc = np.zeros((4, N, N))
    spha[2] = np.pi * 2 / N * np.tile(np.arange(-N / 2, N / 2), N).reshape(N, N, order="F")
    spha[1] = np.pi * 2 / N * np.tile(np.arange(-N / 2, N / 2), (N, 1))
    t = np.arange(N * N, dtype=float).reshape(N, N, order="F")
    im0 = np.random.default_rng(0).uniform(0, 1, (N, N))
    S = mm.sampHighOrder(np.zeros((N, N)), t, spha, conc, grid, None, 1, 0, 0)
    k0 = np.reshape(S * im0, (N, N), order="F")
    k1 = fftnc(im0, 2)
    cost = np.sqrt(np.sum((np.abs(k0) - np.abs(k1)) ** 2)) / k0.size
    assert cost < 1e-6
    im1 = np.reshape(S.H * k0, (N, N), order="F")
    assert np.sqrt(np.sum(np.abs(im1 - im0) ** 2)) / im0.size < 1e-6


def test_highorder_workload_small(mm):
    from matmri_gb300 import synth
    b0, t, spha, conc, grid = synth.highorder_inputs(N=32, M=2048, seed=5)
    S = mm.sampHighOrder(b0, t, spha, conc, grid)
    Sr = ShoRef(b0, t, spha, conc, grid)
    rng = np.random.default_rng(1)
    x = crandn(rng, (32, 32, 4))
    y = crandn(rng, (2048, 4))
    assert rel(S * x, Sr.mtimes(x)) < 1e-5
    assert rel(S.H * y, Sr.H.mtimes(y)) < 1e-5


@pytest.mark.parametrize("ncoil", [1, 3, 6, 16, 21, 40])
@pytest.mark.parametrize("shape", [((24, 20), 1500), ((32, 32), 1024), ((20, 18), 1501)])
def test_tensor_core_contraction(mm, ncoil, shape):
    """The tensor-core paths (FP16 hi + scaled lo splits, FP32 accumulation) against the FP64
    restatement and the SIMT path, both directions: the tcgen05 kernel (default; it reads a
    zero-padded blocked copy of the table, so 1501 samples need no special case) and the mma.sync
    kernel, coil counts across the coil-group widths (8, 16, 32 and two groups of 32) and sizes that
    are not multiples of the 32-input stage, the 128-row tile or the 4-stage phase block."""
    from matmri_gb300 import synth
    imN, M = shape
    b0, t, spha, conc, grid = synth.highorder_inputs(N=imN[0], M=M, seed=11)
    grid = {k: v[:, :imN[1]] for k, v in grid.items()}
    b0 = b0[:, :imN[1]]
    S = mm.sampHighOrder(b0, t, spha, conc, grid)
    Sr = ShoRef(b0, t, spha, conc, grid)
    rng = np.random.default_rng(ncoil)
    x = crandn(rng, list(imN) + [ncoil])
    y = crandn(rng, (M, ncoil))
    yr, xr = Sr.mtimes(x), Sr.H.mtimes(y)
    yt, xt = S * x, S.H * y
    assert rel(yt, yr) < 1e-5
    assert rel(xt, xr) < 1e-5
    S.set_tensor(2)
    assert rel(S * x, yr) < 1e-5
    assert rel(S.H * y, xr) < 1e-5
    S.set_tensor(False)
    assert rel(yt, S * x) < 1e-5
    assert rel(xt, S.H * y) < 1e-5


def test_kbase_property(mm):
    """S.kbase (read by mrSampFuncMat.m:35) equals the FP64 restatement's B @ P, also from a
    setPhiDiv copy, whose kbase is the base encoding's."""
    from matmri_gb300 import synth
    b0, t, spha, conc, grid = synth.highorder_inputs(N=24, M=700, seed=4)
    S = mm.sampHighOrder(b0, t, spha, conc, grid)
    Sr = ShoRef(b0, t, spha, conc, grid)
    kb = S.kbase
    ref = Sr.kbase()
    assert kb.shape == (24 * 24, 700)
    assert np.max(np.abs(kb - ref)) <= 1e-12 * np.max(np.abs(ref))
    S2 = S.setPhiDiv(0.1 * spha, 0.1 * conc)
    assert np.array_equal(S2.kbase, kb)


# ---- approach 1: SVD + NUFFT interpolated encoding (sampHighOrder.m:314-359) ----
def _interp_op(mm, case, grid, mask=None):
    return mm.sampHighOrder(case["b0"], case["t"], case["spha"], case["coco"], grid, mask, 1, 0, 1,
                            {"svdThresh": 0.01, "subFact": 5})


@pytest.mark.parametrize("orient", [0, 1, 2, 3])
def test_interp_vs_restatement_same_factors(mm, orient):
    # the device applies the host-formed factors: forward / adjoint against the FP64 useInterpWorker
    from oracle.sho_interp_ref import ShoInterpRef
    from sho_cases import interp_case, orient_grid
    case = interp_case(32, seed=1)
    grid = orient_grid(case, orient)
    S = _interp_op(mm, case, grid)
    f = dict(kloc=S.traj_kloc, phsShft=S.phsShft, svdTime=S.svdTime, svdSpace=S.svdSpace)
    R = ShoInterpRef([32, 32], f)
    rng = np.random.default_rng(orient)
    x = crandn(rng, (32, 32, 3))
    y = crandn(rng, (case["M"], 3))
    assert rel(S * x, R.mtimes(x)) < 1e-5
    assert rel(S.H * y, R.H.mtimes(y)) < 1e-5


@pytest.mark.parametrize("orient", [0, 2])
def test_interp_reference_criteria(mm, orient):
    # tests.m:127-139 (useSingle branch 149-155: adjoint to 1e-5) and the comparison with the direct encoding
    from sho_cases import interp_case, orient_grid
    case = interp_case(64, seed=1)
    grid = orient_grid(case, orient)
    S = _interp_op(mm, case, grid)
    rng = np.random.default_rng(5)
    x = crandn(rng, (64, 64))
    y = crandn(rng, case["M"])
    Sx, Sy = S * x, S.H * y
    d1 = np.vdot(x.ravel(order="F"), Sy.ravel(order="F"))
    d2 = np.vdot(Sx.ravel(), y)
    assert abs(d1 - d2) / min(abs(d1), abs(d2)) < 1e-5
    direct = ShoRef(case["b0"], case["t"], case["spha"], case["coco"], grid).mtimes(x).ravel()
    assert np.linalg.norm(direct - Sx.ravel()) / direct.size < 1e-4


def test_interp_masked_and_sense_cgne(mm):
    # a b0 mask (sampHighOrder.m:808-818, 854-858) and the encoding inside mrSampFunc + cgne with coils
    from oracle.sense_ref import RcvrRef, cgne_ref, mrsampfunc
    from oracle.sho_interp_ref import ShoInterpRef
    from sho_cases import interp_case, orient_grid
    from matmri_gb300 import synth
    case = interp_case(32, seed=4)
    grid = orient_grid(case, 1)
    mask = (case["x"] ** 2 + case["y"] ** 2) < (0.9 * np.abs(case["x"]).max()) ** 2
    S = _interp_op(mm, case, grid, mask)
    assert np.all(S.svdSpace[~mask.reshape(-1, order="F")] == 0)
    f = dict(kloc=S.traj_kloc, phsShft=S.phsShft, svdTime=S.svdTime, svdSpace=S.svdSpace)
    Sr = ShoInterpRef([32, 32], f)
    maps = synth.coil_maps(32, 4, 1)
    A = mm.mrSampOp(S, mm.rcvrOp(maps, 0))
    Rr = RcvrRef(maps)
    img = synth.ellipse_phantom(32, 6, 2, complex_phase=True)
    data = mrsampfunc(img, "notransp", Sr, Rr)
    assert rel(A(img, "notransp"), data) < 1e-5
    opt = {"xChangeThresh": None, "resThresh": None}
    x, *_ = mm.cgne(A, data, None, 6, opt)
    xr, *_ = cgne_ref(lambda v, tr: mrsampfunc(v, tr, Sr, Rr), data, None, 6, opt)
    assert rel(x, xr) < 1e-4


# ---- setPhiDiv (sampHighOrder.m:590-622; tests.m:42-62) ----
@pytest.mark.parametrize("nd", [1, 2, 3])
def test_phidiv_vs_oracle(mm, nd):
    rng = np.random.default_rng(20 + nd)
    imN = [round(64 ** (2 / nd))] * nd
    kN = [round(64 ** (1 / nd))] * nd
    b0, t, spha, conc, grid = _rand_case(rng, imN, kN)
    zs = np.zeros([16, 1] + kN[1:])
    dspha = np.diff(np.concatenate([zs, spha], axis=1), axis=1)           # tests.m:43-48
    dconc = np.diff(np.concatenate([np.zeros([4, 1] + kN[1:]), conc], axis=1), axis=1)
    S = mm.sampHighOrder(b0, t, spha, conc, grid)
    Sd = S.setPhiDiv(dspha, dconc)
    R = ShoRef(b0, t, spha, conc, grid)
    Rd = R.setPhiDiv(dspha, dconc)
    x = crandn(rng, imN + [3])
    y = crandn(rng, kN + [2])
    ref = Rd.mtimes(x)
    assert rel(Sd * x, ref) < 1e-5
    assert rel(Sd.H * y, R.H.mtimes(y)) < 1e-5          # the adjoint ignores phiDiv
    assert rel(S * x, R.mtimes(x)) < 1e-5               # value semantics: S itself is unchanged


def test_phidiv_inside_sense(mm):
    # forward model of findDelAuto's delay update: mrSampFunc(x, 'notransp', S.setPhiDiv(...), R)
    from matmri_gb300 import synth
    from oracle.sense_ref import RcvrRef, mrsampfunc
    b0, t, spha, conc, grid = synth.highorder_inputs(N=32, M=1024, seed=3)
    dspha = np.gradient(spha, axis=1)
    S = mm.sampHighOrder(b0, t, spha, conc, grid).setPhiDiv(dspha, np.zeros((0, t.size)))
    Rf = ShoRef(b0, t, spha, conc, grid).setPhiDiv(dspha, np.zeros((0, t.size)))
    maps = synth.coil_maps(32, 4, 1)
    img = synth.ellipse_phantom(32, 6, 2, complex_phase=True)
    A = mm.mrSampOp(S, mm.rcvrOp(maps, 0))
    assert rel(A(img, "notransp"), mrsampfunc(img, "notransp", Rf, RcvrRef(maps))) < 1e-5
