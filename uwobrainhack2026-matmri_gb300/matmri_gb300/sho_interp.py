"""Plan of the interpolated ``sampHighOrder`` encoding (approach 1), formed on the host in FP64.

prepForInterp (operators/@sampHighOrder/sampHighOrder.m:700-889) splits the
encoding phase into the in-plane linear terms, which become the sample
locations of a 2D nufftOp plus a phase shift (createNufftForInterp, 624-698),
and a slowly varying remainder ``b`` (prepForDirect on the terms
``[1, 4:end]``, the concomitant terms and B0, 807) whose exponential is
factored by a truncated SVD ``exp(i b) ~ U S V^H`` (825-858).  The factors
are computed on time samples subsampled by ``subFact`` after a Gaussian
smoothing of the coefficients (subSampTime, 959-982) and ``svdTime`` is
filled back with piecewise cubic Hermite interpolation (846-852).

The reference uses ``svds`` for the largest triplets, starting from
``svdNtry`` (default 30) and growing the count by 1.2x until one falls below
``svdThresh * s_1``; it keeps the triplets up to and including that one and
stops with an error past 200 (827-839).  Here small matrices take the exact
LAPACK SVD; larger ones a randomized subspace iteration (Halko, Martinsson
and Tropp, SIAM Review 53(2), 2011, Algorithm 4.4: a Gaussian test matrix,
two power iterations with re-orthonormalisation, oversampling 10) that grows
its rank the same way.  Each triplet's free unit phase is fixed so that the
largest entry of its time vector is real and positive (the Hermite fill-in
of svdTime is not linear, so the result depends on it; ``svds`` leaves it
arbitrary).  The device applies the factors (``csrc/sho_interp.cu``).
"""
from __future__ import annotations

import math

import numpy as np

_EPS = np.finfo(np.float64).eps
EXACT_SVD_MAX = 2048          # min(rows, cols) up to which the exact SVD is taken


def _harm_basis(x, y, z, n):
    """basisFuncHarm.m:24-96 (terms used by the residual phase: 1, 4..16)."""
    r2 = x * x + y * y + z * z
    table = {
        1: lambda: np.ones_like(x), 2: lambda: x, 3: lambda: y, 4: lambda: z,
        5: lambda: x * y, 6: lambda: z * y, 7: lambda: 3 * z * z - r2, 8: lambda: x * z,
        9: lambda: x * x - y * y, 10: lambda: 3 * y * x * x - y ** 3, 11: lambda: x * z * y,
        12: lambda: (5 * z * z - r2) * y, 13: lambda: 5 * z ** 3 - 3 * z * r2,
        14: lambda: (5 * z * z - r2) * x, 15: lambda: x * x * z - y * y * z,
        16: lambda: x ** 3 - 3 * x * y * y,
    }
    if n not in table:
        raise ValueError("interpolated approach: spherical-harmonic terms above 16 are not supported")
    return table[n]()


def _conc_basis(x, y, z, n):
    """basisFuncConc.m:13-23."""
    return {1: lambda: z * z, 2: lambda: x * x + y * y, 3: lambda: x * z, 4: lambda: y * z}[n]()


def _gauss_window(sz, alpha):
    """filtNd(sz, alpha, 1, 'gauss') (general/filtNd.m:49-56), max-normalised."""
    xs = np.arange(-sz / 2, sz / 2) if sz % 2 == 0 else np.arange(-(sz // 2), sz // 2 + 1, dtype=np.float64)
    sig = sz * alpha / 2.355
    w = np.exp(-0.5 * (xs / sig) ** 2)
    return w / w.max()


def _smooth_time(a, win):
    """convn(a, win(:)', 'same') along axis 1 with zero padding (odd window)."""
    h = win.size // 2
    pad = np.zeros((a.shape[0], a.shape[1] + 2 * h) + a.shape[2:])
    pad[:, h:h + a.shape[1]] = a
    out = np.zeros_like(a)
    for k in range(win.size):
        out += win[k] * pad[:, 2 * h - k:2 * h - k + a.shape[1]]
    return out


def subsample_time(spha, conc, t, subfact):
    """subSampTime (sampHighOrder.m:959-982); time along axis 1 of spha/conc, axis 0 of t."""
    M1 = t.shape[0]
    inds = list(range(0, M1, subfact))
    if inds[-1] != M1 - 1:
        inds.append(M1 - 1)
    inds = np.asarray(inds)
    if subfact > 1:
        h = math.ceil(subfact / 2)
        win = _gauss_window(2 * (h + 1), 0.5)[1:]
        win = win / win.sum()
        s2, c2 = _smooth_time(spha, win), _smooth_time(conc, win)
        for src, dst in ((spha, s2), (conc, c2)):
            dst[:, :h] = src[:, :h]
            dst[:, M1 - h:] = src[:, M1 - h:]
        spha, conc = s2, c2
    return spha[:, inds], conc[:, inds], t[inds], inds


def trajectory(gx, gy, gz, spha):
    """createNufftForInterp (sampHighOrder.m:624-698) for axial 2D grids: kloc [M, 2], phsShft [M]."""
    if gx.ndim != 2 or min(gx.shape) < 2:
        raise ValueError("the interpolated approach needs a 2-D grid")
    if gz[1, 1] - gz[0, 0] != 0:
        raise ValueError("non-axial slices not supported for interpolated approach")
    N1, N2 = gx.shape
    if N1 % 2 or N2 % 2:
        raise ValueError("the interpolated approach needs even image sizes (centre index end/2+1)")
    k = np.zeros((spha.shape[1], 2))
    if abs(gx[0, 1] - gx[0, 0]) > _EPS:
        if gy[0, 1] - gy[0, 0] != 0:
            raise ValueError("non-axial slices not supported for interpolated approach")
        r1, r2 = abs(gy[1, 0] - gy[0, 0]), abs(gx[0, 1] - gx[0, 0])
        k[:, 0] = (1.0 if gy[1, 0] - gy[0, 0] > 0 else -1.0) * spha[2] / 2 / np.pi * r1
        k[:, 1] = (1.0 if gx[0, 1] - gx[0, 0] > 0 else -1.0) * spha[1] / 2 / np.pi * r2
        shift = gy[N1 // 2, 0] * spha[2] + gx[0, N2 // 2] * spha[1]
    else:
        r1, r2 = abs(gx[1, 0] - gx[0, 0]), abs(gy[0, 1] - gy[0, 0])
        k[:, 0] = (1.0 if gx[1, 0] - gx[0, 0] > 0 else -1.0) * spha[1] / 2 / np.pi * r1
        k[:, 1] = (1.0 if gy[0, 1] - gy[0, 0] > 0 else -1.0) * spha[2] / 2 / np.pi * r2
        shift = gx[N1 // 2, 0] * spha[1] + gy[0, N2 // 2] * spha[2]
    return k, np.exp(1j * shift)


def residual_phase(x, y, z, b0, mask, t, spha, conc):
    """prepForDirect (sampHighOrder.m:496-588) on the terms [1, 4:end]: b [V, Ms] = B @ P."""
    cols, rows = [], []
    for n in [1] + list(range(4, spha.shape[0] + 1)):
        bf = _harm_basis(x, y, z, n)
        if n > 4 and mask is not None:
            bf = bf * mask
        cols.append(bf)
        rows.append(spha[n - 1])
    for n in range(1, conc.shape[0] + 1):
        bf = _conc_basis(x, y, z, n)
        cols.append(bf * mask if mask is not None else bf)
        rows.append(conc[n - 1])
    if t.size > 1:
        bb = np.zeros_like(x) if b0 is None else b0
        cols.append(bb * mask if mask is not None else bb)
        rows.append(t)
    return np.stack(cols, axis=1) @ np.stack(rows, axis=0)


def _randomized_svd(E, k, rng, power=2, over=10):
    """Randomized subspace iteration (Halko, Martinsson, Tropp 2011, Alg. 4.4)."""
    m, n = E.shape
    r = min(k + over, m, n)
    Om = rng.standard_normal((n, r)) + 1j * rng.standard_normal((n, r))
    Q, _ = np.linalg.qr(E @ Om)
    for _ in range(power):
        W, _ = np.linalg.qr(E.conj().T @ Q)
        Q, _ = np.linalg.qr(E @ W)
    Ub, s, Vh = np.linalg.svd(Q.conj().T @ E, full_matrices=False)
    return Q @ Ub, s, Vh


def _fix_phase(U, Vh):
    """Rotates each triplet so that the largest entry of its time vector is real and positive.

    The SVD leaves a unit phase per triplet free; the piecewise cubic Hermite
    fill-in of svdTime is not linear, so the interpolated encoding depends on
    that phase.  Fixing it makes the factors independent of the SVD method.
    """
    j = np.argmax(np.abs(Vh), axis=1)
    ph = Vh[np.arange(Vh.shape[0]), j]
    ph = ph / np.abs(ph)
    return U * ph[None, :], Vh * np.conj(ph)[:, None]


def truncated_svd(E, thresh, ntry=30, seed=0):
    """Leading triplets of E up to and including the first with s / s_1 < thresh (sampHighOrder.m:825-839)."""
    U, s, Vh = _truncated_svd(E, thresh, ntry, seed)
    U, Vh = _fix_phase(U, Vh)
    return U, s, Vh


def _truncated_svd(E, thresh, ntry, seed):
    if min(E.shape) <= EXACT_SVD_MAX:
        U, s, Vh = np.linalg.svd(E, full_matrices=False)
        below = np.nonzero(s / s[0] < thresh)[0]
        ns = int(below[0]) + 1 if below.size else s.size
        if ns > 200:
            raise ValueError("many large singular values. Try providing mask or adjusting svdThresh.")
        return U[:, :ns], s[:ns], Vh[:ns]
    rng = np.random.default_rng(seed)
    k = int(ntry)
    while True:
        if k > 200:
            raise ValueError("many large singular values. Try providing mask or adjusting svdThresh.")
        U, s, Vh = _randomized_svd(E, k, rng)
        below = np.nonzero(s[:k] / s[0] < thresh)[0]
        if below.size:
            ns = int(below[0]) + 1
            return U[:, :ns], s[:ns], Vh[:ns]
        k = math.ceil(1.2 * k)


def prep_for_interp(b0, sampTimes, phs_spha, phs_conc, grid, b0mask=None, svdThresh=0.05, subFact=5,
                    svdNtry=None):
    """prepForInterp (sampHighOrder.m:700-889), subFactSpc = 1, 2D axial slices.

    Returns dict(kloc [M, 2], phsShft [M], svdTime [M, L], svdSpace [V, L], s [L]).
    """
    gx = np.asarray(grid["x"], dtype=np.float64)
    gy = np.asarray(grid["y"], dtype=np.float64)
    gz = np.asarray(grid["z"], dtype=np.float64)
    t = np.asarray(sampTimes, dtype=np.float64)
    M1 = t.shape[0] if t.ndim > 1 and t.shape[1] > 1 else t.size
    t2 = t.reshape(M1, -1, order="F")
    M = t2.size
    nsp = np.shape(phs_spha)[0]
    sp = np.asarray(phs_spha, dtype=np.float64).reshape(nsp, M1, -1, order="F")
    if phs_conc is None or np.size(phs_conc) == 0:
        pc = np.zeros((0, M1, t2.shape[1]))
    else:
        pc = np.asarray(phs_conc, dtype=np.float64).reshape(np.shape(phs_conc)[0], M1, -1, order="F")
    kloc, shift = trajectory(gx, gy, gz, sp.reshape(nsp, M, order="F"))
    subFact = max(1, int(subFact))
    sps, pcs, ts, inds = subsample_time(sp, pc, t2, subFact)
    Ms = ts.size
    x, y, z = (g.reshape(-1, order="F") for g in (gx, gy, gz))
    bb = None if b0 is None or np.size(b0) == 0 else np.asarray(b0, dtype=np.float64).reshape(-1, order="F")
    mask = None if b0mask is None or np.size(b0mask) == 0 else \
        np.asarray(b0mask, dtype=np.float64).reshape(-1, order="F")
    b = residual_phase(x, y, z, bb, mask, ts.reshape(-1, order="F"), sps.reshape(nsp, Ms, order="F"),
                       pcs.reshape(pcs.shape[0], Ms, order="F"))
    keep = None
    if mask is not None:
        keep = mask > 0.5
        b = b[keep]
    E = np.exp(1j * b)
    del b
    U, s, Vh = truncated_svd(E, svdThresh, 30 if svdNtry is None else svdNtry)
    del E
    L = s.size
    svdTime = Vh.T * s                                   # conj(V S), sampHighOrder.m:845
    if subFact > 1:
        from scipy.interpolate import PchipInterpolator
        st3 = svdTime.reshape(len(inds), t2.shape[1], L, order="F")
        q = np.arange(inds[-1] + 1)
        svdTime = (PchipInterpolator(inds, st3.real, axis=0)(q)
                   + 1j * PchipInterpolator(inds, st3.imag, axis=0)(q)).reshape(M, L, order="F")
    svdSpace = U
    if keep is not None:
        full = np.zeros((x.size, L), dtype=np.complex128)
        full[keep] = U
        svdSpace = full
    return dict(kloc=kloc, phsShft=shift, svdTime=np.ascontiguousarray(svdTime), svdSpace=svdSpace, s=s)
