"""FP64 restatement of MatMRI's ``@nufftOp`` (TEST ORACLE — not the product).

Follows ``operators/@nufftOp/nufftOp.m`` of the reference line by line:
plan construction ``doPrep`` (nufftOp.m:138-274), ``mtimes`` forward
(nufftOp.m:378-394) and adjoint (nufftOp.m:354-377), the Toeplitz mode
(nufftOp.m:348-352, 410-432) and the centered FFT helpers ``fftnc`` /
``ifftnc`` (general/fftnc.m:31-56, general/ifftnc.m:88-113).

Arrays use MATLAB index semantics: an image is ``x[i1, i2, ..., extra...]``
(numpy shape ``(N1, N2, ..., E...)``), samples are ``y[m, extra...]``.
Vectorisation (``x(:)``) is column-major, so reshapes here use ``order='F'``.

Parity pinning: see ``oracle/__init__.py``; this module is pinned by the
reference's own ``@nufftOp/tests.m`` identities (ported in
``tests/test_oracle_nufft.py``).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.fft as sfft
import scipy.sparse as sp

# Threads for the oracle's FFTs (1 for tests; the timed CPU baseline sets all host cores).
FFT_WORKERS = 1


def _max_prime_factor(n: int) -> int:
    f, p = 1, 2
    while p * p <= n:
        while n % p == 0:
            f, n = p, n // p
        p += 1
    return max(f, n) if n > 1 else f


def os_grid_size(imN, os_):
    """Oversampled grid size; nufftOp.m:146-152."""
    osN = [int(math.ceil(n * os_ / 2.0) * 2) for n in imN]
    for d in range(len(osN)):
        while _max_prime_factor(osN[d]) > 7:
            osN[d] += 2
    return osN


def besseli0(z):
    """Modified Bessel function I0 (FP64), power series sum_k (z^2/4)^k/(k!)^2.

    The reference calls MATLAB's ``besseli(0, .)`` (nufftOp.m:164); the
    series converges with positive terms (no cancellation) for the kernel
    arguments used here (0 <= z <= ~25), agreeing with it to ~1e-15.
    """
    z = np.asarray(z, dtype=np.float64)
    q = (z * z) / 4.0
    term = np.ones_like(z)
    acc = np.ones_like(z)
    for k in range(1, 200):
        term = term * q / (k * k)
        acc = acc + term
        if np.all(term <= 1e-17 * acc):
            break
    return acc


def kb_beta(kwidth, os_):
    """Kaiser-Bessel shape parameter; nufftOp.m:155."""
    return math.pi * math.sqrt(kwidth ** 2 / os_ ** 2 * (os_ - 0.5) ** 2 - 0.8)


def kb_table(kwidth, os_):
    """Tabulated KB kernel incl. the trailing zero; nufftOp.m:154-165."""
    precision = 1e-6
    bet = kb_beta(kwidth, os_)
    Nkern = int(math.ceil(0.5 * (kwidth + 1) * math.sqrt(0.37 / os_ ** 2 / precision)) * 2)
    kx = np.linspace(-1.0, 1.0, Nkern)
    kern = np.append(besseli0(bet * np.sqrt(1.0 - kx ** 2)), 0.0)
    kern = kern / kern.sum() * (len(kern) - 2) / kwidth
    return kern, Nkern, bet


def deapod(N, G, kwidth, bet):
    """Deapodisation ``comp{nD}`` for one dim; nufftOp.m:171-181."""
    x = np.arange(-N / 2, N / 2) * math.pi * kwidth / G
    x = np.sqrt(x.astype(np.complex128) ** 2 - bet ** 2)
    c = x / np.sin(x)
    # MATLAB min() of a complex array orders by magnitude; c is real positive here.
    c = c / c[np.argmin(np.abs(c))]
    c = c * math.sqrt(G / N)
    return np.real_if_close(c, tol=1e6).astype(np.complex128)


def fftnc(a, N=None, doShift=1, doScale=1, sz=None):
    """general/fftnc.m:1-56 (forward FFT over the first N dims, unitary scaling)."""
    a = np.asarray(a)
    if N is None:
        N = a.ndim
    N = min(N, a.ndim)
    scale = 1.0
    for n in range(N):
        if doShift:
            a = np.fft.fftshift(a, axes=n)
        a = sfft.fft(a, n=(sz[n] if sz is not None else None), axis=n, workers=FFT_WORKERS)
        if doShift:
            a = np.fft.fftshift(a, axes=n)
        scale *= math.sqrt(a.shape[n])
    if doScale:
        a = a / scale
    return a


def ifftnc(a, N=None, doShift=1, doScale=1, sz=None):
    """general/ifftnc.m:58-113 (inverse FFT over the first N dims, unitary scaling)."""
    a = np.asarray(a)
    if N is None:
        N = a.ndim
    N = min(N, a.ndim)
    scale = 1.0
    for n in range(N):
        if doShift:
            a = np.fft.ifftshift(a, axes=n)
        a = sfft.ifft(a, n=(sz[n] if sz is not None else None), axis=n, workers=FFT_WORKERS)
        if doShift:
            a = np.fft.ifftshift(a, axes=n)
        scale *= math.sqrt(a.shape[n])
    if doScale:
        a = a * scale
    return a


def padcrop(x, sz):
    """Centered zero-pad / crop of the leading dims (general/padcrop.m:28-84).

    Pad: ``floor(npc/2)`` zeros before (padcrop.m:46); crop: start at
    ``floor(npc/2)`` (padcrop.m:66).
    """
    x = np.asarray(x)
    for d, n in enumerate(sz):
        cur = x.shape[d]
        npc = n - cur
        if npc > 0:
            pad = [(0, 0)] * x.ndim
            pad[d] = (npc // 2, npc - npc // 2)
            x = np.pad(x, pad)
        elif npc < 0:
            start = (-npc) // 2
            idx = [slice(None)] * x.ndim
            idx[d] = slice(start, start + n)
            x = x[tuple(idx)]
    return x


class NufftRef:
    """FP64 ``nufftOp`` plan (nufftOp.m:89-136 constructor, 138-274 doPrep)."""

    def __init__(self, imN, kloc, dcf=None, os_=1.5, kwidth=6):
        self.imgN = [int(n) for n in np.atleast_1d(imN)]
        nd = len(self.imgN)
        kloc = np.asarray(kloc, dtype=np.float64).reshape(-1, nd, order="F") if np.ndim(kloc) < 2 \
            else np.asarray(kloc, dtype=np.float64)
        self.kloc = kloc
        self.dcf = None if dcf is None else np.asarray(dcf, dtype=np.float64).reshape(-1)
        self.os = float(os_)
        self.kwidth = int(kwidth)
        self.adjoint = False
        self.isToep = False
        self._prep()

    # nufftOp.m:138-274
    def _prep(self):
        nd = len(self.imgN)
        W = self.kwidth
        kloc_a = self.kloc + 0.5                                     # 141
        self.osN = os_grid_size(self.imgN, self.os)                   # 146-152
        kern, Nkern, bet = kb_table(W, self.os)                       # 154-165
        self.kern, self.Nkern, self.beta = kern, Nkern, bet
        self.comp = [deapod(self.imgN[d], self.osN[d], W, bet) for d in range(nd)]  # 171-186
        M = kloc_a.shape[0]
        offs1 = np.arange(-W / 2 + 1, W / 2 + 1)                      # 192-198 (ndgrid, first dim fastest)
        grids = np.meshgrid(*([offs1] * nd), indexing="ij")
        sampOffsets = [g.reshape(-1, order="F") for g in grids]
        C = np.ones((M, W ** nd))
        for d in range(nd):                                           # 216-227
            kia = kloc_a[:, d] * self.osN[d]
            kia = np.floor(kia) - kia
            for s in range(W ** nd):
                ki = (kia + sampOffsets[d][s]) * (Nkern - 1) / W + Nkern / 2 + 0.5
                frac = ki - np.floor(ki)
                ki = np.floor(ki).astype(np.int64)                    # 1-based index into kern
                C[:, s] *= (1 - frac) * kern[ki - 1] + frac * kern[ki]
        cart = []
        for d in range(nd):                                           # 230-238
            ci = np.floor(kloc_a[:, d] * self.osN[d])[:, None] + sampOffsets[d][None, :] + self.osN[d] / 2 + 1
            ci = np.where(ci > self.osN[d], ci - self.osN[d], ci)
            ci = np.where(ci < 1, ci + self.osN[d], ci)
            cart.append(ci.astype(np.int64) - 1)                      # 0-based
        lin = np.zeros_like(cart[0])                                  # sub2ind, column-major (243-245)
        stride = 1
        for d in range(nd):
            lin = lin + cart[d] * stride
            stride *= self.osN[d]
        rows = np.repeat(np.arange(M)[:, None], W ** nd, axis=1)
        self.convMat = sp.csr_matrix((C.ravel(), (rows.ravel(), lin.ravel())),
                                     shape=(M, int(np.prod(self.osN))))       # 257
        # fftShiftArray (258-273)
        G = self.osN
        fsm = -(np.arange(G[0]) - G[0] / 2) * self.imgN[0] / G[0]
        fsm = fsm.reshape([G[0]] + [1] * (nd - 1))
        for d in range(1, nd):
            shp = [1] * nd
            shp[d] = G[d]
            fsm = fsm - ((np.arange(G[d]) - G[d] / 2) * self.imgN[d] / G[d]).reshape(shp)
        self.fftShiftArray = np.exp(1j * math.pi * fsm)
        self.weights = C
        self.cartInds = lin

    def ctranspose(self):
        """nufftOp.m:276-278 (value-class copy with the adjoint flag flipped)."""
        other = object.__new__(NufftRef)
        other.__dict__.update(self.__dict__)
        other.adjoint = not self.adjoint
        return other

    @property
    def H(self):
        return self.ctranspose()

    def _bcast(self, v, nextra, lead):
        return v.reshape([-1] + [1] * nextra) if lead == 1 else v

    def mtimes(self, x):
        """nufftOp.m:284-408 for a single batch (all extra dims in one matrix op)."""
        x = np.asarray(x)
        nd = len(self.imgN)
        if self.isToep:
            return self._toep_apply(x)
        if self.adjoint:                                                 # 354-377
            M = self.kloc.shape[0]
            extra = x.shape[1:]
            y = x.reshape(M, -1, order="F").astype(np.complex128)
            if self.dcf is not None:
                y = y * self.dcf[:, None]                                # 357
            y = self.convMat.T @ y                                       # 359
            y = y.reshape(list(self.osN) + [-1], order="F")
            y = y * np.conj(self.fftShiftArray)[..., None]               # 362
            y = fftnc(y, nd, doShift=0)                                  # 364
            y = y[tuple(slice(0, n) for n in self.imgN)]                 # 366-372
            for d in range(nd):                                          # 374-377
                shp = [1] * (nd + 1)
                shp[d] = self.imgN[d]
                y = y * self.comp[d].reshape(shp)
            return y.reshape(list(self.imgN) + list(extra), order="F")
        extra = x.shape[nd:]                                             # 378-394
        y = x.reshape(list(self.imgN) + [-1], order="F").astype(np.complex128)
        for d in range(nd):
            shp = [1] * (nd + 1)
            shp[d] = self.imgN[d]
            y = y * self.comp[d].reshape(shp)
        y = ifftnc(y, nd, doShift=0, doScale=1, sz=self.osN)             # 384
        y = y * self.fftShiftArray[..., None]                            # 386
        y = y.reshape(int(np.prod(self.osN)), -1, order="F")
        y = self.convMat @ y                                             # 389
        if self.dcf is not None:
            y = y * self.dcf[:, None]                                    # 392
        return y.reshape([self.kloc.shape[0]] + list(extra), order="F")

    __mul__ = lambda self, x: self.mtimes(x)

    # Toeplitz (nufftOp.m:410-432 prepToep, 348-352 apply)
    def prepToep(self, tos=None, kwidth=None):
        if self.isToep:
            return self
        if tos is None:
            tos = 0.5 * (self.os - 1) + 1                                # 416
        if kwidth is None:
            kwidth = self.kwidth
        S = NufftRef([2 * n for n in self.imgN], self.kloc, self.dcf, tos, kwidth)   # 421
        ones = self.dcf if self.dcf is not None else np.ones(self.kloc.shape[0])
        T = S.ctranspose().mtimes(ones.astype(np.complex128))            # 423/425
        T = (2 ** len(self.imgN)) * ifftnc(T)                            # 427
        other = object.__new__(NufftRef)
        other.__dict__.update(self.__dict__)
        other.toepTF = T
        other.isToep = True
        return other

    def _toep_apply(self, x):
        nd = len(self.imgN)
        extra = x.shape[nd:]
        y = x.reshape(list(self.imgN) + [-1], order="F").astype(np.complex128)
        out = np.empty_like(y)
        for e in range(y.shape[-1]):
            p = padcrop(y[..., e], [2 * n for n in self.imgN])
            p = fftnc(self.toepTF * ifftnc(p, nd), nd)
            out[..., e] = padcrop(p, self.imgN)
        return out.reshape(list(self.imgN) + list(extra), order="F")


def nudft_forward(imN, kloc, x, dcf=None, chunk=2048):
    """Direct FP64 NUDFT with the reference's centering and scaling.

    y_m = dcf_m * c * prod_d N_d^{-1/2} * sum_i x_i exp(+2 pi i sum_d k_{m,d} (i_d - N_d/2))
    with c = exp(i pi sum_d N_d / 2): the constant that the reference's phase
    ramp ``fftShiftArray`` (nufftOp.m:262-271) contributes at grid index 0.
    This is the ground truth that both the restatement and the CUDA path
    report their interpolation error against.
    """
    imN = [int(n) for n in imN]
    nd = len(imN)
    kloc = np.asarray(kloc, dtype=np.float64).reshape(-1, nd)
    M = kloc.shape[0]
    x = np.asarray(x, dtype=np.complex128)
    extra = x.shape[nd:]
    xf = x.reshape(int(np.prod(imN)), -1, order="F")
    grids = np.meshgrid(*[np.arange(n) - n / 2 for n in imN], indexing="ij")
    pos = np.stack([g.reshape(-1, order="F") for g in grids], axis=1)          # [V, nd]
    c = np.exp(1j * math.pi * sum(imN) / 2) / math.sqrt(float(np.prod(imN)))
    y = np.empty((M, xf.shape[1]), dtype=np.complex128)
    for m0 in range(0, M, chunk):
        ph = 2 * math.pi * kloc[m0:m0 + chunk] @ pos.T
        y[m0:m0 + chunk] = np.exp(1j * ph) @ xf
    y *= c
    if dcf is not None:
        y *= np.asarray(dcf, dtype=np.float64).reshape(-1, 1)
    return y.reshape([M] + list(extra), order="F")


def nudft_adjoint(imN, kloc, y, dcf=None, chunk=2048):
    """Adjoint of :func:`nudft_forward` (exact, FP64)."""
    imN = [int(n) for n in imN]
    nd = len(imN)
    kloc = np.asarray(kloc, dtype=np.float64).reshape(-1, nd)
    M = kloc.shape[0]
    y = np.asarray(y, dtype=np.complex128).reshape(M, -1, order="F")
    extra_n = y.shape[1]
    if dcf is not None:
        y = y * np.asarray(dcf, dtype=np.float64).reshape(-1, 1)
    grids = np.meshgrid(*[np.arange(n) - n / 2 for n in imN], indexing="ij")
    pos = np.stack([g.reshape(-1, order="F") for g in grids], axis=1)
    c = np.exp(-1j * math.pi * sum(imN) / 2) / math.sqrt(float(np.prod(imN)))
    V = pos.shape[0]
    x = np.zeros((V, extra_n), dtype=np.complex128)
    for m0 in range(0, M, chunk):
        ph = 2 * math.pi * kloc[m0:m0 + chunk] @ pos.T
        x += np.exp(-1j * ph).T @ y[m0:m0 + chunk]
    x *= c
    return x.reshape(list(imN) + [extra_n], order="F")
