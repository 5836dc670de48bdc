"""Batched uneven cgne (mmr_cgne_solve_batch): every solve of the batch equals the same cgne run alone,
and the FP64 restatement of cgne.m."""
import numpy as np
import pytest

from gpu_util import crandn, rel
from oracle.nufft_ref import NufftRef
from oracle.sense_ref import RcvrRef, cgne_ref, mrsampfunc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mm():
    import matmri_gb300 as m
    return m


def _slices(mm, n=6, seed=0):
    from matmri_gb300 import synth
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        N = int(rng.choice([32, 48, 64]))
        C = int(rng.choice([2, 4, 8]))
        M = int(rng.integers(1500, 4000))
        kloc = rng.uniform(-0.5, 0.5, (M, 2))
        maps = synth.coil_maps(N, C, seed + i)
        A = mm.mrSampOp(mm.nufftOp([N, N], kloc, None, 1, 2.0, 4), mm.rcvrOp(maps, 0))
        y = crandn(rng, (M, C)).astype(np.complex64)
        out.append((A, y, kloc, maps, N))
    return out


@pytest.mark.parametrize("opt", [{"resThresh": None, "xChangeThresh": None}, {"resThresh": 1e-3}])
def test_batch_equals_single_solves(mm, opt):
    sl = _slices(mm)
    xs, infos = mm.cgne_batch([s[0] for s in sl], [s[1] for s in sl], 10, opt)
    for (A, y, _, _, _), x, info in zip(sl, xs, infos):
        x1, res1, _, _, _, _, st1 = mm.cgne(A, y, None, 10, opt)
        assert rel(x, x1) < 1e-6
        assert info["status"] == st1 and info["nit"] == len(res1) - 1
        np.testing.assert_allclose(info["resSqAll"], res1, rtol=1e-5)


def test_batch_matches_fp64_cgne(mm):
    sl = _slices(mm, n=3, seed=5)
    opt = {"resThresh": None, "xChangeThresh": None}
    xs, _ = mm.cgne_batch([s[0] for s in sl], [s[1] for s in sl], 8, opt)
    for (A, y, kloc, maps, N), x in zip(sl, xs):
        Sr, Rr = NufftRef([N, N], kloc, None, 2.0, 4), RcvrRef(maps)
        op = lambda v, t: mrsampfunc(v, t, Sr, Rr)
        xr = cgne_ref(op, y.astype(np.complex128), None, 8, opt)[0]
        assert rel(x, xr) < 1e-4
