"""Generates the golden vectors in this directory from the FP64 oracle.

Run from the repository root:  python tests/golden/make_golden.py
Each case is a small seeded input with the oracle's output (the reference is
MATLAB and cannot be run here; the oracle is pinned to the reference's own
known-answer tests, see tests/test_oracle_*.py).  tests/test_golden.py checks
that the oracle still reproduces these files; tests/test_gpu_golden.py checks
the CUDA path against them.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.bfista_ref import HaarRef, bfista_ref  # noqa: E402
from oracle.nufft_ref import NufftRef  # noqa: E402
from oracle.sense_ref import RcvrRef, cgne_ref, mrsampfunc  # noqa: E402
from oracle.sho_ref import ShoRef  # noqa: E402


def crandn(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def cases():
    out = {}
    for name, imN, M, os_, kw, nb in [("nufft1d", [48], 200, 2.0, 4, 2), ("nufft2d", [32, 40], 700, 2.0, 4, 3),
                                      ("nufft2d_kw6", [32, 32], 600, 1.5, 6, 1), ("nufft3d", [12, 16, 10], 500, 2.0, 4, 1)]:
        rng = np.random.default_rng(len(name) * 31 + M)
        kloc = rng.uniform(-0.5, 0.5, (M, len(imN)))
        dcf = rng.uniform(0.2, 1.0, M)
        S = NufftRef(imN, kloc, dcf, os_, kw)
        x = crandn(rng, imN + [nb])
        y = crandn(rng, (M, nb))
        out[name] = dict(imN=np.array(imN), kloc=kloc, dcf=dcf, os=os_, kw=kw, x=x, y=y,
                         fwd=S.mtimes(x), adj=S.H.mtimes(y))
    # SENSE normal operator and a short cgne
    rng = np.random.default_rng(7)
    N, C, M = 32, 3, 800
    kloc = rng.uniform(-0.5, 0.5, (M, 2))
    maps = crandn(rng, (N, N, C)) * 0.5
    S, R = NufftRef([N, N], kloc, None, 2.0, 4), RcvrRef(maps)
    x = crandn(rng, (N, N))
    data = mrsampfunc(x, "notransp", S, R) + 0.05 * crandn(rng, (M, C))
    normal = mrsampfunc(mrsampfunc(x, "notransp", S, R), "transp", S, R)
    opt = {"xChangeThresh": None, "resThresh": None}
    xc, rs, _, xn, xd, _, st = cgne_ref(lambda v, t: mrsampfunc(v, t, S, R), data, None, 6, opt)
    out["sense"] = dict(kloc=kloc, maps=maps, x=x, data=data, normal=normal, cg_x=xc, cg_res=rs.real,
                        cg_xnorm=xn.real, cg_status=st)
    # sampHighOrder
    rng = np.random.default_rng(11)
    imN, kN = [16, 12], [96]
    b0 = rng.standard_normal(imN)
    t = rng.uniform(0, 1e-2, kN)
    spha = rng.standard_normal([16] + kN) * 3
    conc = rng.standard_normal([4] + kN)
    grid = {k: rng.standard_normal(imN) * 0.5 for k in "xyz"}
    Sh = ShoRef(b0, t, spha, conc, grid)
    xs = crandn(rng, imN + [2])
    ys = crandn(rng, kN + [2])
    out["sho"] = dict(b0=b0, t=t, spha=spha, conc=conc, gx=grid["x"], gy=grid["y"], gz=grid["z"], x=xs, y=ys,
                      fwd=Sh.mtimes(xs), adj=Sh.H.mtimes(ys))
    # Haar bands and bfista
    rng = np.random.default_rng(13)
    xh = crandn(rng, (32, 24))
    W = HaarRef([2, 2], [32, 24])
    out["haar"] = dict(x=xh, bands=np.stack(W.forward(xh), axis=-1))
    xb, rsb, rxb, _, meb = bfista_ref(lambda v, t: mrsampfunc(v, t, S, R), data, HaarRef([2, 2], [N, N]), 0.02,
                                      mrsampfunc(data, "transp", S, R), 8, {"maxEig": 50.0, "resThresh": 0})
    out["bfista"] = dict(x=xb, res=rsb, rx=rxb)
    return out


if __name__ == "__main__":
    for name, d in cases().items():
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
        print("wrote", name)
