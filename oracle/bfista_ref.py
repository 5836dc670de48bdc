"""FP64 restatement of ``bfista``, ``powermethod``, ``softthresh`` and the
undecimated Haar ``dwtND`` used as bfista's regulariser (TEST ORACLE).

* ``softthresh``   — general/softthresh.m:4
* ``powermethod``  — iterativeSolvers/powermethod.m:1-67
* ``HaarRef``      — operators/@dwtND: dwtND.m:28-79 (constructor, db1,
  undecimated), set.family (108-116: filters divided by sqrt(2) when
  undecimated), mtimes.m:1-122 (decomp/recon, decompSep/reconSep band
  ordering), wavConv1D.m:1-44 (object-domain circshift filtering)
* ``bfista_ref``   — iterativeSolvers/bfista.m:1-246

Wavelet coefficients are returned as a list ``[low, high[0][0..2^d-2], ...]``
("bands") in the order waveletObj stores them (low, then high{j}{s}).
Test infrastructure only; see ``oracle/__init__.py``.
"""
from __future__ import annotations

import math

import numpy as np

# MATLAB wfilters('db1'): Lo_D = [1 1]/sqrt(2), Hi_D = [-1 1]/sqrt(2),
# Lo_R = [1 1]/sqrt(2), Hi_R = [1 -1]/sqrt(2).
_S = 1.0 / math.sqrt(2.0)
DB1 = dict(Lo_D=np.array([_S, _S]), Hi_D=np.array([-_S, _S]),
           Lo_R=np.array([_S, _S]), Hi_R=np.array([_S, -_S]))


def softthresh(w, lam):
    """general/softthresh.m:4 — sign(w).*max(abs(w)-lam,0) (complex sign = w/|w|)."""
    w = np.asarray(w)
    a = np.abs(w)
    with np.errstate(invalid="ignore", divide="ignore"):
        sg = np.where(a > 0, w / np.where(a > 0, a, 1), 0)
    return sg * np.maximum(a - lam, 0)


def powermethod(A, x0, NitMax=50, doAtA=1, xdiffThresh=1e-3):
    """iterativeSolvers/powermethod.m:1-67 (A is a callable A(x, transp))."""
    x = np.asarray(x0)
    x_prev = x
    nit = 0
    while True:                                                           # 38-57
        x = A(A(x, "notransp"), "transp") if doAtA else A(x, "notransp")
        x = x / np.linalg.norm(x.reshape(-1))
        xdiff = np.linalg.norm(x.reshape(-1) - x_prev.reshape(-1))
        x_prev = x
        nit += 1
        if xdiff < xdiffThresh or nit >= NitMax:
            break
    AtAx = A(A(x, "notransp"), "transp") if doAtA else A(x, "notransp")  # 60-65
    return np.vdot(x.reshape(-1), AtAx.reshape(-1)) / np.vdot(x.reshape(-1), x.reshape(-1))


class HaarRef:
    """Undecimated db1 dwtND (dwtND(J, imSize, false, 'db1'))."""

    def __init__(self, J, imSize):
        imSize = list(imSize)
        J = list(np.broadcast_to(np.asarray(J), (len(imSize),)))
        self.J = [0 if imSize[d] == 1 else int(J[d]) for d in range(len(imSize))]   # dwtND.m:55
        self.imSize = imSize
        f = {k: v / math.sqrt(2.0) for k, v in DB1.items()}              # dwtND.m:111-116
        self.Lo_D, self.Hi_D, self.Lo_R, self.Hi_R = f["Lo_D"], f["Hi_D"], f["Lo_R"], f["Hi_R"]

    def _conv(self, x, filt, j, dim, recon):
        """wavConv1D.m:22-43 (non-Fourier, undecimated)."""
        y = 0
        L = len(filt)
        for n in range(L):
            shift = n
            if recon:
                shift = shift - L + 1
            shift = (2 ** (j - 1)) * shift
            if filt[n] != 0:
                y = y + filt[n] * np.roll(x, -shift, axis=dim)            # circshift(x,-shift,dim)
        return y

    def decomp(self, x):
        """mtimes.m:32-51 + decompSep 74-96. Returns (low, high) with high[j-1] a list."""
        low = np.asarray(x, dtype=np.complex128)
        high = []
        for j in range(1, max(self.J) + 1):
            dec = [self.J[d] >= j for d in range(len(self.J))]
            hj = [None] * (2 ** sum(dec) - 1)
            ds = 0
            for d in range(len(dec)):
                if dec[d]:
                    hj[2 ** ds - 1] = self._conv(low, self.Hi_D, j, d, 0)
                    for s in range(1, 2 ** ds):
                        hj[2 ** ds + s - 1] = self._conv(hj[s - 1], self.Hi_D, j, d, 0)
                        hj[s - 1] = self._conv(hj[s - 1], self.Lo_D, j, d, 0)
                    low = self._conv(low, self.Lo_D, j, d, 0)
                    ds += 1
            high.append(hj)
        return low, high

    def recon(self, low, high):
        """mtimes.m:53-72 + reconSep 98-122."""
        low = np.asarray(low, dtype=np.complex128)
        high = [list(h) for h in high]
        for j in range(max(self.J), 0, -1):
            rec = [self.J[d] >= j for d in range(len(self.J))]
            hj = high[j - 1]
            ds = sum(rec) - 1
            for d in range(len(rec) - 1, -1, -1):
                if rec[d]:
                    low = self._conv(low, self.Lo_R, j, d, 1)
                    low = low + self._conv(hj[2 ** ds - 1], self.Hi_R, j, d, 1)
                    for s in range(1, 2 ** ds):
                        hj[s - 1] = self._conv(hj[s - 1], self.Lo_R, j, d, 1) + \
                            self._conv(hj[2 ** ds + s - 1], self.Hi_R, j, d, 1)
                    ds -= 1
        return low

    def to_bands(self, low, high):
        return [low] + [b for hj in high for b in hj]

    def from_bands(self, bands):
        low = bands[0]
        high, i = [], 1
        for j in range(1, max(self.J) + 1):
            n = 2 ** sum(self.J[d] >= j for d in range(len(self.J))) - 1
            high.append(list(bands[i:i + n]))
            i += n
        return low, high

    def forward(self, x):
        return self.to_bands(*self.decomp(x))

    def adjoint(self, bands):
        return self.recon(*self.from_bands(bands))


def bfista_ref(A, bin, R, lam, x0=None, NitMax=200, opt=None):
    """iterativeSolvers/bfista.m:1-246 with R an undecimated Haar (HaarRef).

    ``A`` is a callable ``A(x, transp)``; ``lam`` is a scalar or a per-band
    list (the waveletObj lambda of demos/demo_wavelet.m:101-102).
    Returns ``(x, resSqAll, RxAll, testAll, maxEig)``.
    """
    o = dict(maxEig=None, resThresh=1e-5, gtruth=None, xMask=None, nRestart=NitMax + 1)
    if opt:
        o.update(opt)
    if x0 is None:
        x0 = A(bin, "transp")                                            # 73-75
    maxEig = o["maxEig"] if o["maxEig"] is not None else powermethod(A, x0)   # 81-89
    stepSz = 0.9 / (2 * abs(maxEig))                                     # 90
    y = x0
    resSqAll = np.zeros(NitMax + 1)
    RxAll = np.zeros(NitMax + 1)
    testAll = np.zeros((NitMax + 1, 2))
    nbands = len(R.forward(np.zeros(R.imSize)))
    lams = list(lam) if isinstance(lam, (list, tuple, np.ndarray)) else [lam] * nbands
    nit, nitToRestart, t_prev, x_prev = 1, 1, 1.0, x0
    while True:                                                           # 127-233
        residual_y = A(y, "notransp") - bin
        grad = 2 * A(residual_y, "transp")
        resSqAll[nit - 1] = np.real(np.vdot(residual_y.reshape(-1), residual_y.reshape(-1)))
        g = y - stepSz * grad
        wb = R.forward(g)
        RxAll[nit - 1] = sum(np.sum(np.abs(lams[i] * wb[i])) for i in range(nbands))   # 146-148
        wb = [softthresh(wb[i], lams[i] * stepSz) for i in range(nbands)]              # 149
        x = R.adjoint(wb)                                                               # 150
        if o["xMask"] is not None:
            x = x * o["xMask"]
        xdiff = x - x_prev                                                              # 195-197
        t = 0.5 * (1 + math.sqrt(1 + 4 * t_prev ** 2))
        y = x + (t_prev - 1) / t * xdiff
        t_prev = t
        x_prev = x
        finished = nit >= NitMax
        testVal = None
        if nit > 1:                                                                     # 208-222
            c = resSqAll[:nit] + RxAll[:nit]
            tv = np.abs(np.diff(c)) / (resSqAll[nit - 1] + RxAll[nit - 1])
            i1 = max(1, nit - 3)
            testVal = float(np.mean(tv[i1 - 1:]))
            testAll[nit - 1, 0] = testVal
            testAll[nit - 1, 1] = np.real(np.vdot(xdiff.reshape(-1), xdiff.reshape(-1))) / \
                np.real(np.vdot(x.reshape(-1), x.reshape(-1)))
        if nit > 1 and testVal < o["resThresh"]:
            finished = True
        nit += 1
        nitToRestart += 1
        if nitToRestart >= o["nRestart"]:
            nitToRestart = 1
            t_prev = 1.0
        if finished:
            break
    n = nit - 1
    testAll = testAll[:n].copy()
    testAll[0, :] = np.nan
    return x, resSqAll[:n], RxAll[:n], testAll, maxEig
