"""The CUDA path against the committed golden vectors (tests/golden/), through
the C ABI: per-application rel-L2 <= 1e-5, cgne/bfista images <= 1e-4."""
import os

import numpy as np
import pytest

from gpu_util import rel

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(HERE, f"{name}.npz"))


@pytest.fixture(scope="module")
def mm():
    import matmri_gb300 as m
    return m


@pytest.mark.parametrize("name", ["nufft1d", "nufft2d", "nufft2d_kw6", "nufft3d"])
def test_nufft_golden(mm, name):
    g = load(name)
    N = mm.nufftOp(list(g["imN"]), g["kloc"], g["dcf"], 1, float(g["os"]), int(g["kw"]))
    assert rel(N * g["x"], g["fwd"]) < 1e-5
    assert rel(N.H * g["y"], g["adj"]) < 1e-5


def test_sense_and_cgne_golden(mm):
    g = load("sense")
    S = mm.nufftOp([32, 32], g["kloc"], None, 1, 2.0, 4)
    A = mm.mrSampOp(S, mm.rcvrOp(g["maps"], 0))
    assert rel(A.normal(g["x"]), g["normal"]) < 1e-5
    x, rs, _, xn, _, _, st = mm.cgne(A, g["data"], None, 6, {"xChangeThresh": None, "resThresh": None})
    assert rel(x, g["cg_x"]) < 1e-4 and st == int(g["cg_status"])
    assert np.allclose(rs, g["cg_res"], rtol=1e-3)


def test_sho_golden(mm):
    g = load("sho")
    grid = {"x": g["gx"], "y": g["gy"], "z": g["gz"]}
    S = mm.sampHighOrder(g["b0"], g["t"], g["spha"], g["conc"], grid)
    assert rel(S * g["x"], g["fwd"]) < 1e-5
    assert rel(S.H * g["y"], g["adj"]) < 1e-5


def test_haar_and_bfista_golden(mm):
    g = load("haar")
    bands = mm.dwtND([2, 2], [32, 24]) * g["x"]
    assert rel(np.stack(bands, axis=-1), g["bands"]) < 1e-6
    s, b = load("sense"), load("bfista")
    S = mm.nufftOp([32, 32], s["kloc"], None, 1, 2.0, 4)
    A = mm.mrSampOp(S, mm.rcvrOp(s["maps"], 0))
    x0 = A(s["data"], "transp")
    x, rs, rx, _, _ = mm.bfista(A, s["data"], mm.dwtND([2, 2], [32, 32]), 0.02, x0, 8,
                                {"maxEig": 50.0, "resThresh": 0})
    assert rel(x, b["x"]) < 1e-4
    assert np.allclose(rs, b["res"], rtol=1e-3) and np.allclose(rx, b["rx"], rtol=1e-3)
