"""Seeded inputs of the interpolated-encoding test of @sampHighOrder/tests.m:66-139.

A radial trajectory of N0 - 4 spokes x 2 N0 samples stands in for
``projection(N0, N0 - 4, 2)``; sample times are 1..M; the grid is shifted by
(+3, -2) pixels with pixel sizes 0.8 / 0.95; B0 is a random fifth-order
polynomial scaled to pi / t_end; every term but the in-plane linear ones is a
random quartic in time with amplitude 0.05 of the linear phase at half the
field of view (eddy currents), and the concomitant terms likewise.
"""
import numpy as np


def interp_case(N0=32, seed=1):
    rng = np.random.default_rng(seed)
    rn = rng.standard_normal
    ns, nr = N0 - 4, 2 * N0
    ang = np.arange(ns) * np.pi / ns
    r = (np.arange(nr) - nr / 2) / nr
    kloc = np.stack([np.outer(np.cos(ang), r).ravel(), np.outer(np.sin(ang), r).ravel()], 1)
    M = kloc.shape[0]
    t = np.arange(1, M + 1, dtype=np.float64)
    xg, yg = np.meshgrid(np.arange(-N0 / 2, N0 / 2), np.arange(-N0 / 2, N0 / 2))
    dx, dy = 0.8, 0.95
    kloc[:, 0] = 2 * np.pi * kloc[:, 0] / np.abs(kloc[:, 0]).max() / 2 / dx
    kloc[:, 1] = 2 * np.pi * kloc[:, 1] / np.abs(kloc[:, 1]).max() / 2 / dy
    x = (xg + 3) * dx
    y = (yg - 2) * dy
    scl = 0.5 * np.abs(x).max()
    b0 = (scl ** 5 * (rn() * x + rn() * y)
          + scl * (rn() * x ** 4 + rn() * x ** 3 * y + rn() * x ** 2 * y ** 2 + rn() * x * y ** 3 + rn() * y ** 4)
          + rn() * x ** 5 + rn() * x ** 4 * y + rn() * x ** 3 * y ** 2 + rn() * x ** 2 * y ** 3
          + rn() * x * y ** 4 + rn() * y ** 5)
    b0 = b0 / np.abs(b0).max() * np.pi / t[-1]
    sclt = 0.5 * t[-1]
    quartic = lambda: rn() + 2 * rn() / sclt * t + rn() / sclt ** 2 * t ** 2 + rn() / sclt ** 3 * t ** 3 \
        + rn() / sclt ** 4 * t ** 4
    spha = np.zeros((16, M))
    coco = np.zeros((4, M))
    spha[1:3] = kloc.T
    for n in [1] + list(range(4, 17)):
        a = quartic()
        if 1 < n < 5:
            a = 0.05 * a / scl
        elif 1 < n < 10:
            a = 0.05 * a / scl ** 2
        elif n >= 10:
            a = 0.05 * a / scl ** 3
        spha[n - 1] += a
    for n in range(4):
        coco[n] = 0.05 * quartic() / scl ** 2
    return dict(b0=b0, t=t, spha=spha, coco=coco, x=x, y=y, scl=scl, M=M, N0=N0)


def orient_grid(c, orient):
    """The four grid orientations of @sampHighOrder/tests.m:102-115."""
    x, y = c["x"], c["y"]
    gx, gy = [(x, y), (x.T, y.T), (-x, -y), (-x.T, -y.T)][orient]
    return dict(x=gx, y=gy, z=c["scl"] * np.ones_like(x))


def finddel_case(N=24, C=4, M=1536, true_delay=0.37, seed=7, snr=200.0, turns=3, wobble=2.0):
    """A delay-estimation problem for findDelAuto (findDel/findDelAuto.m): the inputs of
    synth.finddel_inputs with data simulated by the FP64 direct encoding at the exact phases of
    t + true_delay, through the coil maps, plus complex Gaussian noise at the given SNR."""
    from oracle.sense_ref import RcvrRef
    from oracle.sho_ref import ShoRef
    from matmri_gb300 import synth
    rng = np.random.default_rng(seed)
    c = synth.finddel_inputs(N, C, M, turns, wobble, seed)
    dt = c["datatime"]
    S = ShoRef(c["b0"], dt, c["phases"](dt + true_delay).T, np.zeros((4, M)), c["grid"])
    data = S.mtimes(RcvrRef(c["maps"]).mtimes(c["img"]))
    sig = np.sqrt(np.mean(np.abs(data) ** 2)) / snr
    data = data + sig * (rng.standard_normal(data.shape) + 1j * rng.standard_normal(data.shape)) / np.sqrt(2)
    c.update(data=data, true_delay=true_delay)
    return c
