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
    """A delay-estimation problem for findDelAuto (findDel/findDelAuto.m).

    Data times are 20..20+M-1 (unit dwell); the field trajectory is tabulated
    every 0.5 from t = 0 and the data are simulated with the exact phases at
    t + true_delay (FP64 direct encoding, coil maps, complex Gaussian noise at
    the given SNR).  The trajectory is a 3-turn spiral in the linear terms, a
    constant term and two small second-order terms.
    """
    from oracle.sense_ref import RcvrRef
    from oracle.sho_ref import ShoRef
    from matmri_gb300 import synth
    rng = np.random.default_rng(seed)
    fov = 0.22
    c = (np.arange(N) - N / 2) * fov / N
    X, Y = np.meshgrid(c, c, indexing="ij")
    grid = {"x": X, "y": Y, "z": np.zeros_like(X)}
    T = 20 + M + 40
    kmax = np.pi * N / fov

    def phases(t):
        tau = t / T
        r = kmax * tau
        th = 2 * np.pi * turns * tau
        sp = np.zeros((t.size, 16))
        sp[:, 0] = wobble * np.sin(2 * np.pi * 8 * tau)
        sp[:, 1] = r * np.cos(th)
        sp[:, 2] = r * np.sin(th)
        sp[:, 4] = 40.0 * tau ** 2
        sp[:, 8] = -25.0 * tau
        return sp

    tdwell = 0.5
    lenTraj = int(T / tdwell) + 1
    traj = phases(tdwell * np.arange(lenTraj))
    conc = np.zeros((lenTraj, 4))
    datatime = 20.0 + np.arange(M, dtype=np.float64)
    b0 = 2e-3 * np.exp(-((X - 0.03) ** 2 + (Y + 0.02) ** 2) / 0.004)      # rad per time unit
    maps = synth.coil_maps(N, C, seed)
    img = synth.ellipse_phantom(N, 6, seed + 1, complex_phase=True)
    S = ShoRef(b0, datatime, phases(datatime + true_delay).T, np.zeros((4, M)), grid)
    data = S.mtimes(RcvrRef(maps).mtimes(img))
    sig = np.sqrt(np.mean(np.abs(data) ** 2)) / snr
    data = data + sig * (rng.standard_normal(data.shape) + 1j * rng.standard_normal(data.shape)) / np.sqrt(2)
    return dict(data=data, tdwell=tdwell, traj=traj, conc=conc, datatime=datatime, grid=grid, b0=b0,
                maps=maps, true_delay=true_delay)
