"""FP64 restatement of ``@sampHighOrder`` approach 1, the SVD + NUFFT interpolated
encoding (TEST ORACLE).

* ``filtnd_gauss``     — general/filtNd.m:1-56 (1-D 'gauss' window)
* ``subsamp_time``     — sampHighOrder.m:959-982 (subSampTime)
* ``nufft_for_interp`` — sampHighOrder.m:624-698 (createNufftForInterp, 2-D axial)
* ``prep_for_interp``  — sampHighOrder.m:700-889 (prepForInterp; subFactSpc = 1,
  no SMS slices)
* ``ShoInterpRef``     — sampHighOrder.m:314-359 (useInterpWorker) on an FP64
  ``NufftRef`` trajectory operator (nufftOp defaults os 1.5, kwidth 6).

The encoding matrix less the in-plane linear terms, ``exp(i b)`` with ``b``
from prepForDirect on the terms ``[1, 4:end]`` (sampHighOrder.m:807), is
factored as ``U S V^H``; the reference calls ``svds`` for the largest
singular triplets and keeps them up to and including the first one below
``svdThresh * s_1`` (sampHighOrder.m:825-839).  The oracle takes the exact
LAPACK SVD, whose leading triplets are the ones ``svds`` converges to, and
fixes each triplet's free unit phase so that the largest entry of its time
vector is real and positive (``svds`` leaves that phase arbitrary, and the
Hermite fill-in below is not linear, so the encoding depends on it).
Time-subsampled ``svdTime`` is filled back with piecewise cubic Hermite
interpolation (MATLAB ``interp1(..., 'pchip')``, sampHighOrder.m:846-852),
applied to the real and imaginary parts separately.
Test infrastructure only; see ``oracle/__init__.py``.
"""
from __future__ import annotations

import math

import numpy as np

from .nufft_ref import NufftRef
from .sho_ref import basis_conc, basis_harm

MATLAB_EPS = 2.220446049250313e-16


def filtnd_gauss(sz: int, alpha: float) -> np.ndarray:
    """filtNd(sz, alpha, 1, 'gauss') (filtNd.m:49-56, normalised to max 1 at 37)."""
    if sz % 2 == 0:
        xs = np.arange(-sz / 2, sz / 2)
    else:
        h = sz // 2
        xs = np.arange(-h, h + 1, dtype=np.float64)
    sig = sz * alpha / 2.355
    w = np.exp(-0.5 * (xs / sig) ** 2) / (sig * math.sqrt(2 * math.pi))
    return w / w.max()


def subsamp_time(phs_spha, phs_conc, t, subfact):
    """subSampTime (sampHighOrder.m:959-982).

    phs_spha [n, M1, M2], phs_conc [nc, M1, M2], t [M1, M2]; time runs along
    axis 1 of the coefficient arrays (axis 0 of t).  Returns the smoothed,
    subsampled coefficients, the subsampled times and the kept indices.
    """
    M1 = t.shape[0]
    inds = list(range(0, M1, subfact))                                   # 960
    if inds[-1] != M1 - 1:                                               # 961-964
        inds.append(M1 - 1)
    inds = np.asarray(inds)
    sp, cc = phs_spha.copy(), phs_conc.copy()
    if subfact > 1:                                                      # 968-979
        h = math.ceil(subfact / 2)
        win = filtnd_gauss(2 * (h + 1), 0.5)
        win = win[1:] / win[1:].sum()
        sp = _conv_same(phs_spha, win)
        cc = _conv_same(phs_conc, win)
        sp[:, :h] = phs_spha[:, :h]
        cc[:, :h] = phs_conc[:, :h]
        sp[:, M1 - h:] = phs_spha[:, M1 - h:]
        cc[:, M1 - h:] = phs_conc[:, M1 - h:]
    return sp[:, inds], cc[:, inds], t[inds], inds


def _conv_same(a, win):
    """convn(a, win(:)', 'same') along axis 1 (odd-length window, zero padding)."""
    K = win.size
    h = K // 2
    out = np.zeros_like(a)
    M1 = a.shape[1]
    for k in range(K):
        s = h - k                       # out[j] += a[j + s] * win[k]
        lo, hi = max(0, -s), min(M1, M1 - s)
        if lo < hi:
            out[:, lo:hi] += a[:, lo + s:hi + s] * win[k]
    return out


def nufft_for_interp(grid, phs_spha, kshape):
    """createNufftForInterp (sampHighOrder.m:624-698) for axial 2-D grids.

    Returns kloc [M, 2] (nufftOp sample locations) and phsShft [M] complex.
    """
    gx, gy, gz = (np.asarray(grid[c], dtype=np.float64) for c in ("x", "y", "z"))
    if gx.ndim != 2 or gx.shape[0] < 2 or gx.shape[1] < 2:
        raise ValueError("interpolated approach needs a 2-D grid")
    if gz[1, 1] - gz[0, 0] != 0:                                         # 640-642
        raise ValueError("non-axial slices not supported for interpolated approach")
    sp = phs_spha.reshape(phs_spha.shape[0], -1)
    N1, N2 = gx.shape
    kloc = np.zeros((2, sp.shape[1]))
    if abs(gx[0, 1] - gx[0, 0]) > MATLAB_EPS:                           # 643-663
        if gy[0, 1] - gy[0, 0] != 0:
            raise ValueError("non-axial slices not supported for interpolated approach")
        res1, res2 = abs(gy[1, 0] - gy[0, 0]), abs(gx[0, 1] - gx[0, 0])
        kloc[0] = (1 if gy[1, 0] - gy[0, 0] > 0 else -1) * sp[2] / 2 / math.pi * res1
        kloc[1] = (1 if gx[0, 1] - gx[0, 0] > 0 else -1) * sp[1] / 2 / math.pi * res2
        shft = gy[N1 // 2, 0] * sp[2] + gx[0, N2 // 2] * sp[1]
    else:                                                                # 664-681
        res1, res2 = abs(gx[1, 0] - gx[0, 0]), abs(gy[0, 1] - gy[0, 0])
        kloc[0] = (1 if gx[1, 0] - gx[0, 0] > 0 else -1) * sp[1] / 2 / math.pi * res1
        kloc[1] = (1 if gy[0, 1] - gy[0, 0] > 0 else -1) * sp[2] / 2 / math.pi * res2
        shft = gx[N1 // 2, 0] * sp[1] + gy[0, N2 // 2] * sp[2]
    return kloc.T.copy(), np.exp(1j * shft)                               # 694-695


def residual_phase(grid, b0, t, phs_spha, phs_conc, b0mask, spha_inds):
    """prepForDirect (sampHighOrder.m:496-588) on a subset of spherical-harmonic terms."""
    x = np.asarray(grid["x"], dtype=np.float64).reshape(-1, order="F")
    y = np.asarray(grid["y"], dtype=np.float64).reshape(-1, order="F")
    z = np.asarray(grid["z"], dtype=np.float64).reshape(-1, order="F")
    V = x.size
    tt = np.asarray(t, dtype=np.float64).reshape(-1, order="F")
    sp = phs_spha.reshape(phs_spha.shape[0], tt.size, order="F")
    cc = phs_conc.reshape(phs_conc.shape[0], tt.size, order="F")
    mask = None if b0mask is None else np.asarray(b0mask, dtype=np.float64).reshape(-1, order="F")
    phs = np.zeros((V, sp.shape[1]))
    for n in spha_inds:                                                  # 560-569
        bf = basis_harm(x, y, z, n)
        if n > 4 and mask is not None:
            bf = bf * mask
        phs += bf[:, None] * sp[n - 1][None, :]
    for n in range(1, cc.shape[0] + 1):                                  # 570-579
        bf = basis_conc(x, y, z, n)
        if mask is not None:
            bf = bf * mask
        phs += bf[:, None] * cc[n - 1][None, :]
    if tt.size > 1:                                                      # 580-586
        bb = np.zeros(V) if b0 is None else np.asarray(b0, dtype=np.float64).reshape(-1, order="F")
        if mask is not None:
            bb = bb * mask
        phs += bb[:, None] * tt[None, :]
    return phs


def _pchip_cols(xk, yk, xq):
    from scipy.interpolate import PchipInterpolator
    return PchipInterpolator(xk, yk, axis=0)(xq)


def prep_for_interp(b0, sampTimes, phs_spha, phs_conc, grid, b0mask=None, svdThresh=0.05, subFact=5):
    """prepForInterp (sampHighOrder.m:700-889) with subFactSpc = 1.

    Returns dict(kloc [M,2], phsShft [M], svdTime [M,L], svdSpace [V,L], s [L]).
    """
    t = np.asarray(sampTimes, dtype=np.float64)
    kshape = t.shape if t.ndim > 1 and t.shape[1] > 1 else (t.size,)
    t2 = t.reshape(kshape[0], -1, order="F")
    M = t2.size
    sp = np.asarray(phs_spha, dtype=np.float64).reshape(np.shape(phs_spha)[0], kshape[0], -1, order="F")
    pc = np.zeros((0, kshape[0], t2.shape[1])) if phs_conc is None or np.size(phs_conc) == 0 else \
        np.asarray(phs_conc, dtype=np.float64).reshape(np.shape(phs_conc)[0], kshape[0], -1, order="F")
    kloc, phsShft = nufft_for_interp(grid, sp.reshape(sp.shape[0], -1, order="F"), kshape)
    subFact = max(1, int(subFact))
    sps, pcs, ts, inds = subsamp_time(sp, pc, t2, subFact)              # 780
    spha_inds = [1] + list(range(4, sp.shape[0] + 1))                    # strtIndSpha = 4 (2-D)
    b = residual_phase(grid, b0, ts, sps, pcs, b0mask, spha_inds)       # 807
    V = b.shape[0]
    keep = None
    if b0mask is not None:                                               # 808-818
        keep = np.asarray(b0mask, dtype=np.float64).reshape(-1, order="F") > 0.5
        b = b[keep]
    E = np.exp(1j * b)                                                   # 819
    U, s, Vh = np.linalg.svd(E, full_matrices=False)
    below = np.nonzero(s / s[0] < svdThresh)[0]
    Ns = int(below[0]) + 1 if below.size else s.size                     # 839
    U, s, Vh = U[:, :Ns], s[:Ns], Vh[:Ns]
    for l in range(Ns):      # unit phase: largest entry of each time vector real and positive
        j = int(np.argmax(np.abs(Vh[l])))
        ph = Vh[l, j] / abs(Vh[l, j])
        U[:, l] *= ph
        Vh[l] *= np.conj(ph)
    svdTime = (Vh[:Ns].T * s[:Ns])                                       # 845: conj(V S)
    if subFact > 1:                                                      # 847-852
        st3 = svdTime.reshape(len(inds), t2.shape[1], Ns, order="F")
        q = np.arange(inds[-1] + 1)
        re = _pchip_cols(inds, st3.real, q)
        im = _pchip_cols(inds, st3.imag, q)
        svdTime = (re + 1j * im).reshape(M, Ns, order="F")
    svdSpace = U[:, :Ns]
    if keep is not None:                                                 # 854-858
        full = np.zeros((V, Ns), dtype=np.complex128)
        full[keep] = svdSpace
        svdSpace = full
    return dict(kloc=kloc, phsShft=phsShft.reshape(-1, order="F"), svdTime=svdTime, svdSpace=svdSpace, s=s[:Ns])


class ShoInterpRef:
    """useInterpWorker (sampHighOrder.m:314-359) in FP64 for given factors."""

    def __init__(self, imSize, factors, os_=1.5, kwidth=6):
        self.imSize = list(imSize)
        self.f = factors
        self.traj = NufftRef(self.imSize, factors["kloc"], None, os_, kwidth)
        self.adjoint = False

    def ctranspose(self):
        o = ShoInterpRef.__new__(ShoInterpRef)
        o.__dict__.update(self.__dict__)
        o.adjoint = not self.adjoint
        return o

    @property
    def H(self):
        return self.ctranspose()

    def mtimes(self, x):
        """Forward: x [imSize, extra] -> [M, extra]; adjoint: [M, extra] -> [imSize, extra]."""
        x = np.asarray(x)
        if self.adjoint:
            extra = list(x.shape[1:])
            return self._apply(x).reshape(self.imSize + extra, order="F")
        extra = list(x.shape[len(self.imSize):])
        return self._apply(x).reshape([self.f["svdTime"].shape[0]] + extra, order="F")

    def _apply(self, x):
        f = self.f
        V = int(np.prod(self.imSize))
        sS, sT, ph = f["svdSpace"], f["svdTime"], f["phsShft"]
        M, L = sT.shape
        if self.adjoint:                                                  # 321-338
            yv = np.asarray(x, dtype=np.complex128).reshape(M, -1, order="F")
            R = yv.shape[1]
            u = yv[:, :, None] * np.conj(sT)[:, None, :]                 # 326
            u = np.conj(ph)[:, None, None] * u                           # 327
            img = self.traj.H.mtimes(u.reshape(M, R * L, order="F"))     # 334
            img = img.reshape(V, R, L, order="F")
            out = (img * np.conj(sS)[:, None, :]).sum(axis=2)            # 335-336
            return out
        xv = np.asarray(x, dtype=np.complex128).reshape(V, -1, order="F")   # 338-355
        R = xv.shape[1]
        a = xv[:, :, None] * sS[:, None, :]                               # 344
        a = a.reshape(self.imSize + [R * L], order="F")
        t = self.traj.mtimes(a).reshape(M, R, L, order="F")               # 345
        t = ph[:, None, None] * t                                         # 351
        return (t * sT[:, None, :]).sum(axis=2)                           # 352-353

    __mul__ = lambda self, x: self.mtimes(x)
