"""Seeded synthetic MRI inputs with the shapes of the benchmark workloads.

No public dataset is named for these workloads and the reference's own
image/coil/B0 blobs are not distributed, so every input is generated here
from ``numpy.random.Generator(PCG64(seed))``:

* random-ellipse phantoms (optionally with a smooth complex phase),
* variable-density multi-interleave spirals ``k(tau) = 0.5 tau^1.5 e^{i(2 pi T tau + 2 pi j / n_int)}``,
  ``T = N / (2 n_int R)`` turns, clipped to ``|k| < 0.5``,
* ring-of-Gaussians coil maps with linear phase, root-sum-of-squares
  normalised (the pattern of simulation/simRcvrSens.m:77-79),
* analytic ``|k|`` density compensation (the spiral analogue of
  trajectory/projection.m:15-16),
* complex Gaussian noise at a given SNR,
* high-order encoding inputs: spherical-harmonic phase time courses whose
  non-linear terms are smooth cubics in time at +-5 % of the linear-term
  phase at the FOV edge, a sum-of-Gaussians B0 map spanning +-100 Hz, and a
  30 ms readout.

Arrays follow MATLAB index semantics (image ``[N1, N2]``, samples ``[M]``,
coil maps ``[N1, N2, C]``).
"""
from __future__ import annotations

import math

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(int(seed)))


def ellipse_phantom(N: int, n_ellipses: int = 10, seed: int = 0, complex_phase: bool = False) -> np.ndarray:
    g = rng(seed)
    c = (np.arange(N) - N / 2) / (N / 2)                      # normalised coords in [-1, 1)
    X, Y = np.meshgrid(c, c, indexing="ij")
    img = np.zeros((N, N))
    for _ in range(n_ellipses):
        cx, cy = g.uniform(-0.6, 0.6, 2)
        a, b = g.uniform(0.05, 0.45, 2)
        th = g.uniform(0, math.pi)
        val = g.uniform(0, 1)
        xr = (X - cx) * math.cos(th) + (Y - cy) * math.sin(th)
        yr = -(X - cx) * math.sin(th) + (Y - cy) * math.cos(th)
        img += val * ((xr / a) ** 2 + (yr / b) ** 2 <= 1.0)
    img = img.astype(np.complex128)
    if complex_phase:
        co = g.uniform(-1, 1, 6)
        ph = co[0] + co[1] * X + co[2] * Y + co[3] * X * Y + co[4] * X ** 2 + co[5] * Y ** 2
        ph = ph / max(np.abs(ph).max(), 1e-12) * (math.pi / 2)
        img = img * np.exp(1j * ph)
    return img


def spiral(N: int, n_int: int, samples: int, R: float = 1.0) -> np.ndarray:
    """kloc [n_int*samples, 2] in [-0.5, 0.5), interleave-major (MATLAB kloc(:, [kx ky]))."""
    T = N / (2.0 * n_int * R)
    tau = np.arange(samples) / samples
    ks = []
    for j in range(n_int):
        k = 0.5 * tau ** 1.5 * np.exp(1j * (2 * math.pi * T * tau + 2 * math.pi * j / n_int))
        r = np.abs(k)
        k = np.where(r >= 0.5, k / np.maximum(r, 1e-30) * np.nextafter(0.5, 0), k)
        ks.append(k)
    k = np.concatenate(ks)
    kl = np.stack([k.real, k.imag], axis=1)
    return np.clip(kl, -0.5, np.nextafter(0.5, 0))


def spiral_dcf(kloc: np.ndarray, N: int) -> np.ndarray:
    r = np.sqrt((kloc ** 2).sum(axis=1))
    d = np.maximum(r, 0.5 / N)
    return d / d.max()


def coil_maps(N: int, C: int, seed: int = 0, randomize: bool = False) -> np.ndarray:
    g = rng(seed)
    fov = 1.0
    c = (np.arange(N) - N / 2) / N * fov
    X, Y = np.meshgrid(c, c, indexing="ij")
    radius = 0.6 * fov / 2
    sigma = 0.35 * fov
    maps = np.empty((N, N, C), dtype=np.complex128)
    for ci in range(C):
        rr = radius * (g.uniform(0.8, 1.2) if randomize else 1.0)
        ss = sigma * (g.uniform(0.8, 1.2) if randomize else 1.0)
        ang = 2 * math.pi * ci / C
        cx, cy = rr * math.cos(ang), rr * math.sin(ang)
        mag = np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * ss ** 2))
        a, b = g.uniform(-math.pi, math.pi, 2) / fov
        c0 = g.uniform(-math.pi, math.pi)
        maps[:, :, ci] = mag * np.exp(1j * (a * X + b * Y + c0))
    rss = np.sqrt((np.abs(maps) ** 2).sum(axis=2, keepdims=True))
    return maps / rss


def _grid_torch(N, scale, device):
    import torch
    c = (torch.arange(N, dtype=torch.float64, device=device) - N / 2) / scale
    X, Y = torch.meshgrid(c, c, indexing="ij")
    return X, Y


def ellipse_phantom_torch(N: int, n_ellipses: int = 10, seed: int = 0, complex_phase: bool = False,
                          device="cuda"):
    """``ellipse_phantom`` evaluated with torch on `device` (same draws; complex64 [N, N], column-major)."""
    import torch
    g = rng(seed)
    X, Y = _grid_torch(N, N / 2, device)
    img = torch.zeros((N, N), dtype=torch.float64, device=device)
    for _ in range(n_ellipses):
        cx, cy = g.uniform(-0.6, 0.6, 2)
        a, b = g.uniform(0.05, 0.45, 2)
        th = g.uniform(0, math.pi)
        val = g.uniform(0, 1)
        xr = (X - cx) * math.cos(th) + (Y - cy) * math.sin(th)
        yr = -(X - cx) * math.sin(th) + (Y - cy) * math.cos(th)
        img += val * ((xr / a) ** 2 + (yr / b) ** 2 <= 1.0).to(torch.float64)
    out = img.to(torch.complex128)
    if complex_phase:
        co = g.uniform(-1, 1, 6)
        ph = co[0] + co[1] * X + co[2] * Y + co[3] * X * Y + co[4] * X ** 2 + co[5] * Y ** 2
        ph = ph / max(float(ph.abs().max()), 1e-12) * (math.pi / 2)
        out = out * torch.exp(1j * ph)
    return out.to(torch.complex64).T.contiguous().T


def coil_maps_torch(N: int, C: int, seed: int = 0, randomize: bool = False, device="cuda"):
    """``coil_maps`` evaluated with torch on `device` (same draws; complex64 [N, N, C], column-major)."""
    import torch
    g = rng(seed)
    fov = 1.0
    X, Y = _grid_torch(N, N / fov, device)
    radius, sigma = 0.6 * fov / 2, 0.35 * fov
    maps = torch.empty((C, N, N), dtype=torch.complex128, device=device)
    for ci in range(C):
        rr = radius * (g.uniform(0.8, 1.2) if randomize else 1.0)
        ss = sigma * (g.uniform(0.8, 1.2) if randomize else 1.0)
        ang = 2 * math.pi * ci / C
        cx, cy = rr * math.cos(ang), rr * math.sin(ang)
        mag = torch.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * ss ** 2))
        a, b = g.uniform(-math.pi, math.pi, 2) / fov
        c0 = g.uniform(-math.pi, math.pi)
        maps[ci] = mag * torch.exp(1j * (a * X + b * Y + c0))
    maps = maps / torch.sqrt((maps.abs() ** 2).sum(dim=0, keepdim=True))
    # [C, N1, N2] -> column-major [N1, N2, C]
    return maps.to(torch.complex64).permute(0, 2, 1).contiguous().permute(2, 1, 0)


def add_noise(y: np.ndarray, snr: float, seed: int) -> np.ndarray:
    g = rng(seed)
    sig = math.sqrt(np.mean(np.abs(y) ** 2)) / snr
    return y + sig / math.sqrt(2) * (g.standard_normal(y.shape) + 1j * g.standard_normal(y.shape))


def highorder_inputs(N: int = 128, M: int = 16384, fov: float = 0.22, readout: float = 30e-3,
                     seed: int = 3000, n_int: int = 1):
    """Inputs for ``sampHighOrder``: b0 [N,N] rad/s, t [M] s, phs_spha [16,M], phs_conc [4,M], grid."""
    g = rng(seed)
    c = (np.arange(N) - N / 2) * fov / N
    X, Y = np.meshgrid(c, c, indexing="ij")
    grid = {"x": X, "y": Y, "z": np.zeros_like(X)}
    kl = spiral(N, n_int, M // n_int, 1.0)
    t = np.linspace(0.0, readout, M)
    spha = np.zeros((16, M))
    spha[1] = kl[:, 0] * 2 * math.pi * N / fov
    spha[2] = kl[:, 1] * 2 * math.pi * N / fov
    lin_edge = np.abs(spha[1:3]).max() * (fov / 2)           # linear-term phase at the FOV edge (rad)
    tn = t / readout
    edge = fov / 2
    # basisFuncHarm orders: n=1 (0th), 2-4 (1st), 5-9 (2nd), 10-16 (3rd)
    order = [0, 1, 1, 1, 2, 2, 2, 2, 2, 3, 3, 3, 3, 3, 3, 3]
    for n in range(16):
        if n in (1, 2):
            continue
        co = g.uniform(-1, 1, 4)
        poly = co[0] + co[1] * tn + co[2] * tn ** 2 + co[3] * tn ** 3
        poly = poly / max(np.abs(poly).max(), 1e-12)
        spha[n] = poly * 0.05 * lin_edge / (edge ** order[n])
    conc = np.zeros((4, M))
    b0 = np.zeros((N, N))
    for _ in range(int(g.integers(3, 6))):
        cx, cy = g.uniform(-0.6, 0.6, 2) * fov / 2
        s = g.uniform(0.1, 0.3) * fov
        b0 += g.uniform(-1, 1) * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s ** 2))
    b0 = b0 - b0.min()
    b0 = b0 / max(b0.max(), 1e-12) * 200.0 - 100.0         # +-100 Hz
    b0 = 2 * math.pi * b0                                    # rad/s
    return b0, t, spha, conc, grid


# --- named workloads ---------------------------------------------------------------

def regridding_case(seed: int = 1000):
    """128^2 single-coil regridding: 16 x 2048 spiral, kwidth 4, os 2, |k| DCF, SNR 50."""
    N = 128
    img = ellipse_phantom(N, 10, seed)
    kloc = spiral(N, 16, 2048, 1.0)
    dcf = spiral_dcf(kloc, N)
    return dict(N=N, img=img, kloc=kloc, dcf=dcf, os=2.0, kwidth=4, snr=50.0, seed=seed)


def sense_case(N: int = 256, C: int = 32, n_int: int = 4, samples: int = 4096, R: float = 4.0,
               seed: int = 2000, snr: float | None = None, randomize_coils: bool = False):
    """256^2 x 32-coil CG-SENSE: 4 x 4096 spiral at R = 4, kwidth 4, os 2, complex phantom."""
    img = ellipse_phantom(N, 10, seed, complex_phase=True)
    kloc = spiral(N, n_int, samples, R)
    maps = coil_maps(N, C, seed + 1, randomize=randomize_coils)
    return dict(N=N, C=C, img=img, kloc=kloc, maps=maps, os=2.0, kwidth=4, snr=snr, seed=seed)


def batched_cases(n_slices: int = 64, seed: int = 4000):
    """64 uneven slices: N in {96,128,192,256}, C in {8,16,32}, 2-8 interleaves x 2048-4096 samples."""
    g = rng(seed)
    out = []
    for s in range(n_slices):
        N = int(g.choice([96, 128, 192, 256]))
        C = int(g.choice([8, 16, 32]))
        n_int = int(g.integers(2, 9))
        samples = int(g.integers(2048, 4097))
        out.append(sense_case(N, C, n_int, samples, R=max(1.0, 16.0 / n_int), seed=seed + 10 * s + 1))
    return out


def finddel_inputs(N: int = 24, C: int = 4, M: int = 1536, turns: float = 3.0, wobble: float = 6.0,
                   seed: int = 7, fov: float = 0.22):
    """Inputs of a delay-estimation problem (findDelAuto): data times 20..20+M-1 (unit dwell), a field
    trajectory tabulated every 0.5 from t = 0 (a `turns`-turn spiral in the linear terms, a zeroth-order
    phase oscillation of amplitude `wobble` rad and two small second-order terms), B0, coil maps and an
    ellipse image.  `phases(t)` gives the exact coefficients [t.size, 16] at any time, so that data can be
    simulated at t + delay."""
    c = (np.arange(N) - N / 2) * fov / N
    X, Y = np.meshgrid(c, c, indexing="ij")
    grid = {"x": X, "y": Y, "z": np.zeros_like(X)}
    T = 20 + M + 40
    kmax = math.pi * N / fov

    def phases(t):
        tau = np.asarray(t, dtype=np.float64) / T
        r = kmax * tau
        th = 2 * math.pi * turns * tau
        sp = np.zeros((tau.size, 16))
        sp[:, 0] = wobble * np.sin(2 * math.pi * 8 * tau)
        sp[:, 1] = r * np.cos(th)
        sp[:, 2] = r * np.sin(th)
        sp[:, 4] = 40.0 * tau ** 2
        sp[:, 8] = -25.0 * tau
        return sp

    tdwell = 0.5
    lenTraj = int(T / tdwell) + 1
    return dict(tdwell=tdwell, traj=phases(tdwell * np.arange(lenTraj)), conc=np.zeros((lenTraj, 4)),
                datatime=20.0 + np.arange(M, dtype=np.float64), grid=grid,
                b0=2e-3 * np.exp(-((X - 0.03) ** 2 + (Y + 0.02) ** 2) / 0.004),
                maps=coil_maps(N, C, seed), img=ellipse_phantom(N, 6, seed + 1, complex_phase=True),
                phases=phases)
