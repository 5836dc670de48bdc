"""mrSampFuncMat (dense normal matrix on the device) and the demo's direct solve
against the FP64 restatement (operators/mrSampFuncMat.m, demos/demo_denseMat.m)."""
import numpy as np
import pytest

from gpu_util import crandn, rel

pytestmark = pytest.mark.gpu


def _case(N=24, M=900, C=4, seed=1):
    from matmri_gb300 import synth
    b0, t, spha, conc, grid = synth.highorder_inputs(N=N, M=M, seed=seed)
    maps = synth.coil_maps(N, C, seed + 1)
    rng = np.random.default_rng(seed)
    y = crandn(rng, (M, C))
    return y, maps, b0, t, spha, conc, grid


@pytest.mark.parametrize("masked", [False, True])
def test_dense_normal_vs_restatement(masked):
    import matmri_gb300 as mm
    from oracle.densemat_ref import mrsampfuncmat_ref
    y, maps, b0, t, spha, conc, grid = _case()
    mask = None
    if masked:
        X, Y = grid["x"], grid["y"]
        mask = X ** 2 + Y ** 2 < (0.45 * 0.22) ** 2
    AtA, Aty = mm.mrSampFuncMat(y, maps, b0, t, spha, conc, grid, mask)
    Ar, br = mrsampfuncmat_ref(y, maps, b0, t, spha, conc, grid, mask)
    A = AtA.cpu().numpy()
    assert A.shape == Ar.shape
    assert np.linalg.norm(A - Ar) / np.linalg.norm(Ar) < 1e-5
    assert rel(Aty.cpu().numpy(), br) < 1e-5
    assert np.linalg.norm(A - A.conj().T) / np.linalg.norm(A) < 1e-6


def test_dense_matrix_matches_device_normal_operator():
    # full mask: AtA x == R'S'SR x through the iterative operators (demo_denseMat.m compares the two paths)
    import torch
    import matmri_gb300 as mm
    y, maps, b0, t, spha, conc, grid = _case(N=32, M=1200, C=3, seed=5)
    AtA, _ = mm.mrSampFuncMat(y, maps, b0, t, spha, conc, grid)
    A = mm.mrSampOp(mm.sampHighOrder(b0, t, spha, conc, grid), mm.rcvrOp(maps, 0))
    x = crandn(np.random.default_rng(2), (32, 32))
    ref = A(A(x, "notransp"), "transp").reshape(-1, order="F")
    got = (AtA @ torch.from_numpy(x.reshape(-1, order="F").astype(np.complex64)).cuda()).cpu().numpy()
    assert rel(got, ref) < 1e-5


@pytest.mark.parametrize("lam2", [1e-2, 1.0])
def test_dense_solve_vs_numpy(lam2):
    import matmri_gb300 as mm
    y, maps, b0, t, spha, conc, grid = _case(N=20, M=800, C=4, seed=3)
    AtA, Aty = mm.mrSampFuncMat(y, maps, b0, t, spha, conc, grid)
    x, method = mm.dense_solve(AtA, Aty, lam2)
    A = AtA.cpu().numpy().astype(np.complex128)
    ref = np.linalg.solve(A + lam2 * np.eye(A.shape[0]), Aty.cpu().numpy().astype(np.complex128))
    assert method == "chol"
    assert rel(x.cpu().numpy(), ref) < 1e-4
    # AtA itself is left unchanged (the demo reuses it for every lam2)
    assert np.array_equal(AtA.cpu().numpy(), A.astype(np.complex64))


def test_dense_solve_lu_fallback():
    # an indefinite Hermitian matrix is not Cholesky-factorable: LU with pivoting takes over
    import torch
    import matmri_gb300 as mm
    rng = np.random.default_rng(8)
    n = 64
    Q, _ = np.linalg.qr(crandn(rng, (n, n)))
    d = np.linspace(-2, 3, n)
    d[np.abs(d) < 0.1] = 0.5
    H = (Q * d) @ Q.conj().T
    b = crandn(rng, n)
    Ht = torch.from_numpy(np.ascontiguousarray(H.T).astype(np.complex64)).cuda().T   # column-major storage
    x, method = mm.dense_solve(Ht, torch.from_numpy(b.astype(np.complex64)).cuda(), 0.0)
    assert method == "lu"
    assert rel(x.cpu().numpy(), np.linalg.solve(H, b)) < 1e-4
