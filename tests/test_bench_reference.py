"""The reference arm's CPU solver: mrSampFunc with the coils split over host threads is the FP64
restatement's arithmetic (same values as oracle.sense_ref.mrsampfunc), a solve through it is
cgne_ref's solve, and both bench arms describe the workload with the same config."""
import importlib.util
import os

import numpy as np

from oracle.nufft_ref import NufftRef
from oracle.sense_ref import CoilParallelSense, RcvrRef, cgne_ref, mrsampfunc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _case(N=32, C=6, M=900, seed=3):
    rng = np.random.default_rng(seed)
    kloc = rng.uniform(-0.5, 0.5, (M, 2))
    maps = rng.standard_normal((N, N, C)) + 1j * rng.standard_normal((N, N, C))
    img = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    return kloc, maps, img


def test_coil_parallel_sense_equals_restatement():
    kloc, maps, img = _case()
    S = NufftRef([32, 32], kloc, None, 2.0, 4)
    R = RcvrRef(maps)
    for threads in (1, 4, 6, 16):
        A = CoilParallelSense(S, maps, threads)
        y = A(img, "notransp")
        np.testing.assert_allclose(y, mrsampfunc(img, "notransp", S, R), rtol=0, atol=1e-12)
        x = A(y, "transp")
        ref = mrsampfunc(y, "transp", S, R)
        assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-13
        A.close()


def test_coil_parallel_cgne_equals_restatement():
    kloc, maps, img = _case(C=5)
    S = NufftRef([32, 32], kloc, None, 2.0, 4)
    R = RcvrRef(maps)
    A = CoilParallelSense(S, maps, 3)
    y = A(img, "notransp")
    opt = {"xChangeThresh": None, "resThresh": None}
    x1, r1, *_ = cgne_ref(A, y, None, 6, opt)
    x2, r2, *_ = cgne_ref(lambda v, t: mrsampfunc(v, t, S, R), y, None, 6, opt)
    A.close()
    assert np.linalg.norm(x1 - x2) / np.linalg.norm(x2) < 1e-12
    np.testing.assert_allclose(r1.real, r2.real, rtol=1e-11)


def test_both_arms_share_the_workload_config():
    spec = importlib.util.spec_from_file_location("bench_cfg", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    cfg = b.config_dict(1)
    assert cfg["workload"] == b.WORKLOAD and cfg["coils"] == 32 and cfg["samples"] == 16384
    assert cfg["iterations"] == 30 and cfg["grid"] == [512, 512]
    assert b.config_dict(4)["parallelism"] == "replicas x4"
