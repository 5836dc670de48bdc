"""FP64 restatement of ``@rcvrOp``, ``mrSampFunc``, ``cgne`` and helpers (TEST ORACLE).

* ``RcvrRef``      — operators/@rcvrOp/rcvrOp.m:104-159 (forward ``x.*maps``,
  adjoint ``sum(x.*conj(maps), nDim+1)``).
* ``mrsampfunc``   — operators/mrSampFunc.m:1-160.
* ``cgne_ref``     — iterativeSolvers/cgne.m:1-358 (all stopping rules, W,
  Tikhonov ``gam``/``R``, the explicit-residual restart, history vectors).
* ``CoilParallelSense`` — ``mrSampFunc(x, transp, S, R)`` for a nufftOp S and
  an rcvrOp R with the coils split over host threads: the same FP64 arithmetic
  as ``mrsampfunc``, used to time the reference algorithm on all host cores.

Test infrastructure only; see ``oracle/__init__.py``.
"""
from __future__ import annotations

import math

import numpy as np

from .nufft_ref import fftnc, ifftnc


class RcvrRef:
    """rcvrOp with precomputed maps (rcvrOp.m:47-94 with isCalDat = 0)."""

    def __init__(self, maps):
        self.maps = np.asarray(maps, dtype=np.complex128)
        self.nDim = self.maps.ndim - 1                      # rcvrOp.m:91
        self.adjoint = False

    def ctranspose(self):
        o = RcvrRef.__new__(RcvrRef)
        o.__dict__.update(self.__dict__)
        o.adjoint = not self.adjoint
        return o

    @property
    def H(self):
        return self.ctranspose()

    def mtimes(self, x):
        x = np.asarray(x)
        if self.adjoint:                                     # rcvrOp.m:148-150
            return np.sum(x * np.conj(self.maps), axis=self.nDim)
        return x[..., None] * self.maps if x.ndim == self.nDim else x * self.maps   # rcvrOp.m:152

    __mul__ = lambda self, x: self.mtimes(x)


def mrsampfunc(x, transp, samplingOp, R=None, opt=None):
    """operators/mrSampFunc.m:1-160 (nufftOp / sampHighOrder / Cartesian mask)."""
    opt = dict(opt or {})
    imNFull = opt.get("imNFull")
    daNFull = opt.get("daNFull")
    tikReg = opt.get("tikReg")
    sumDims = opt.get("sumDims")
    hardReal = opt.get("hardReal") or 0
    W = opt.get("W")
    if tikReg is not None and (imNFull is None or daNFull is None):
        raise ValueError("Tikhonov regularization requires opt.imNFull and opt.daNFull")
    is_op = hasattr(samplingOp, "mtimes")
    if transp == "notransp":                                             # 83-120
        if hardReal:
            x = np.real(x)
        if tikReg is not None:
            tr = np.atleast_1d(tikReg)
            x_tik = tr[0] * np.real(x) + 1j * tr[1] * np.imag(x) if tr.size == 2 else tr[0] * x
        if imNFull is not None:
            x = np.reshape(x, imNFull, order="F")
        if R is not None:
            x = R.mtimes(x)
        if sumDims:
            for d in sumDims:
                x = np.sum(x, axis=d - 1, keepdims=True)
        if is_op:
            x = samplingOp.mtimes(x)
        else:
            m = np.asarray(samplingOp)
            nDim = m.ndim if not (m.ndim == 2 and m.shape[1] == 1) else 1
            x = m.reshape(m.shape + (1,) * (x.ndim - m.ndim)) * ifftnc(x, nDim)
        if daNFull is not None:
            x = x.reshape(-1, order="F")
        if tikReg is not None:
            x = np.concatenate([x, x_tik.reshape(-1, order="F")])
        return x
    # transp (121-159)
    if tikReg is not None:
        nda = int(np.prod(daNFull))
        x_tik = x[nda:]
        x = x[:nda]
    if W is not None:
        x = mtimes_bcast(W, x)
    if daNFull is not None:
        x = np.reshape(x, daNFull, order="F")
    if is_op:
        x = samplingOp.ctranspose().mtimes(x)
    else:
        m = np.asarray(samplingOp)
        nDim = m.ndim if not (m.ndim == 2 and m.shape[1] == 1) else 1
        x = fftnc(m.reshape(m.shape + (1,) * (x.ndim - m.ndim)) * x, nDim)
    if R is not None:
        x = R.ctranspose().mtimes(x)
    if imNFull is not None:
        x = x.reshape(-1, order="F")
    if tikReg is not None:
        tr = np.atleast_1d(tikReg)
        x_tik = tr[0] * np.real(x_tik) + 1j * tr[1] * np.imag(x_tik) if tr.size == 2 else tr[0] * x_tik
        x = x + x_tik
    if hardReal:
        x = np.real(x)
    return x


class CoilParallelSense:
    """``opFunc = @(x, transp) mrSampFunc(x, transp, S, R)`` (mrSampFunc.m:83-159,
    rcvrOp.m:144-157, nufftOp.m:354-394) with the coil dimension split into
    contiguous groups that host threads process independently.

    Each coil's forward ``S*(x.*maps_c)`` and adjoint ``S'*y_c`` is exactly the
    restatement's (``NufftRef.mtimes`` on that group's columns, FFTs with one
    worker per thread); the adjoint's coil sum adds the groups' partial sums in
    group order.  numpy, scipy.fft and scipy.sparse release the GIL in their
    kernels, so the groups run concurrently.  Timing use only (the reference's
    MATLAB path uses its host cores the same way through its built-ins).
    """

    def __init__(self, S, maps, threads):
        from concurrent.futures import ThreadPoolExecutor
        self.S, self.SH = S, S.ctranspose()
        self.maps = np.asarray(maps, dtype=np.complex128)
        C = self.maps.shape[-1]
        self.threads = max(1, min(int(threads), C))
        edges = np.linspace(0, C, self.threads + 1).round().astype(int)
        self.groups = [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]
        self.pool = ThreadPoolExecutor(len(self.groups))

    def _fwd(self, x, g):
        a, b = g
        return self.S.mtimes(x[..., None] * self.maps[..., a:b])

    def _adj(self, y, g):
        a, b = g
        return np.sum(self.SH.mtimes(y[:, a:b]) * np.conj(self.maps[..., a:b]), axis=-1)

    def __call__(self, x, transp):
        x = np.asarray(x)
        if transp == "notransp":
            parts = list(self.pool.map(lambda g: self._fwd(x, g), self.groups))
            return np.concatenate(parts, axis=1)
        parts = list(self.pool.map(lambda g: self._adj(x, g), self.groups))
        out = parts[0]
        for q in parts[1:]:
            out = out + q
        return out

    def close(self):
        self.pool.shutdown()


def mtimes_bcast(w, a):
    """MATLAB implicit expansion of ``w .* a`` where ``w`` is a column vector
    (e.g. per-sample weights [M x 1] against data [M x C])."""
    w = np.asarray(w)
    a = np.asarray(a)
    if w.ndim == 1 and a.ndim > 1 and w.shape[0] == a.shape[0]:
        w = w.reshape((-1,) + (1,) * (a.ndim - 1))
    return w * a


def _asub(Ain):
    """cgne.m:343-358 — object (numel==1) or elementwise mask."""
    if hasattr(Ain, "mtimes"):
        return lambda x, t: Ain.mtimes(x) if t == "notransp" else Ain.ctranspose().mtimes(x)
    if np.isscalar(Ain) or np.size(Ain) == 1:
        a = complex(np.asarray(Ain).reshape(-1)[0])
        return lambda x, t: a * x if t == "notransp" else np.conj(a) * x
    A = np.asarray(Ain)
    return lambda x, t: A * x if t == "notransp" else np.conj(A) * x


def _vdot(a, b):
    return complex(np.vdot(np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)))


CGNE_DEFAULTS = dict(resThresh=1e-10, resChangeThresh=None, xChangeThresh=1e-10, expResN=100,
                     nseThreshFact=1.0, nseExtraIt=4, stopOnResInc=0, resIncThresh=1.0,
                     stopOnXdifInc=0, noiseVar=None, gtruth=None)


def cgne_ref(Ain, bin, x0=None, NitMax=None, opt=None, gam=None, Rin=None, W=None,
             nargout=7, noise=None):
    """iterativeSolvers/cgne.m:1-341, FP64.

    ``opt`` keys absent from the dict take cgne.m's defaults (22-89); a key
    present with value ``None`` is MATLAB's ``[]`` (the rule disabled).
    ``noise`` optionally supplies the synthetic noise vector of cgne.m:151-157
    (MATLAB draws it with ``randn``), so that the device solver can be fed the
    same draw.  Returns ``(x, resSqAll, mseAll, xnormAll, xdiffAll, stopThresh, status)``.
    """
    o = dict(CGNE_DEFAULTS)
    if opt:
        o.update(opt)
    if NitMax is None:
        NitMax = 1000                                                    # 22-25
    if gam is not None and not isinstance(gam, (list, tuple)) and np.all(np.asarray(gam) == 0):
        gam = None                                                       # 91-93
    if gam is None:
        Rin = None
    findxnorm = (nargout > 3) or (o["xChangeThresh"] is not None)        # 101-108
    findxdiff = (nargout > 4) or (o["xChangeThresh"] is not None) or (o["stopOnXdifInc"] > 0)
    A = Ain if callable(Ain) and not hasattr(Ain, "mtimes") else _asub(Ain)   # 111-115
    if Rin is not None:
        R = [(_asub(r) if not callable(r) or hasattr(r, "mtimes") else r) for r in Rin] \
            if isinstance(Rin, (list, tuple)) else (_asub(Rin) if not callable(Rin) or hasattr(Rin, "mtimes") else Rin)
    gl = gam if isinstance(gam, (list, tuple)) else None

    def tik(v):
        out = 0
        if gam is None:
            return out
        if isinstance(R, list):
            for nR in range(len(R)):
                out = out + gl[nR] * R[nR](R[nR](v, "notransp"), "transp")
        else:
            out = out + gam * R(R(v, "notransp"), "transp")
        return out

    def normal(v):
        av = A(v, "notransp")
        if W is not None:
            av = mtimes_bcast(W, av)
        return A(av, "transp")

    b = A(mtimes_bcast(W, bin) if W is not None else bin, "transp")                   # 136-140
    if x0 is None:
        x0 = b                                                           # 143-145
    stopThresh = None
    if o["noiseVar"] is not None and o["noiseVar"] > 0:                  # 148-162
        if noise is None:
            rng = np.random.default_rng(0)
            if np.iscomplexobj(bin):
                noise = math.sqrt(o["noiseVar"] / 2) * (rng.standard_normal(np.shape(bin))
                                                         + 1j * rng.standard_normal(np.shape(bin)))
            else:
                noise = math.sqrt(o["noiseVar"]) * rng.standard_normal(np.shape(bin))
        nse = A(noise, "transp")
        stopThresh = o["nseThreshFact"] * _vdot(nse, nse).real
    xold = x0
    res = b - normal(xold)                                               # 164-170
    if gam is not None:
        res = res - tik(xold)                                            # 171-179
    p = res
    res_sq_old = _vdot(res, res)
    nit = 0
    resSqAll = np.zeros(NitMax + 1, dtype=np.complex128)
    resSqAll[0] = res_sq_old
    xnormAll = np.zeros(NitMax + 1, dtype=np.complex128)
    if findxnorm:
        xnormAll[0] = _vdot(x0, x0)
    xdiffAll = np.zeros(NitMax + 1, dtype=np.complex128)
    if findxdiff:
        xdiffAll[0] = xnormAll[0]
    mseAll = np.zeros(NitMax + 1, dtype=np.complex128)
    if o["gtruth"] is not None:
        t = np.asarray(o["gtruth"]).reshape(-1) - np.asarray(x0).reshape(-1)
        mseAll[0] = _vdot(t, t)
    finished = False
    resIncsTotal = 0
    xdifIncsTotal = 0
    lastxdifInc = 0
    status = 0
    while not finished:                                                  # 213-336
        Ap = normal(p)
        if gam is not None:
            Ap = Ap + tik(p)
        alph = res_sq_old / _vdot(p, Ap)                                 # 228
        x = xold + alph * p                                              # 229
        if nit % o["expResN"] == 0:                                      # 230-246
            res = b - normal(x)
            if gam is not None:
                res = res - tik(x)
            betaFact = 0
        else:
            res = res - alph * Ap                                        # 248
            betaFact = 1
        res_sq_new = _vdot(res, res)                                     # 252
        resSqAll[nit + 1] = res_sq_new
        if findxnorm:
            xnormAll[nit + 1] = _vdot(x, x)
        if findxdiff:
            xd = x - xold
            xdiffAll[nit + 1] = _vdot(xd, xd)
        if o["gtruth"] is not None:
            t = np.asarray(o["gtruth"]).reshape(-1) - np.asarray(x).reshape(-1)
            mseAll[nit + 1] = _vdot(t, t)
        if o["xChangeThresh"] is not None and xdiffAll[nit + 1].real < o["xChangeThresh"]:   # 286-290
            finished, status = True, 10
        if o["resThresh"] is not None and res_sq_new.real < o["resThresh"]:                  # 291-295
            finished, status = True, 1
        if o["resChangeThresh"] is not None and abs((resSqAll[nit + 1] - resSqAll[nit]) / resSqAll[nit]) < o["resChangeThresh"]:
            finished, status = True, 2                                                       # 296-300
        if stopThresh is not None and res_sq_new.real < stopThresh:                          # 301-307
            NitMax = nit + o["nseExtraIt"]
            stopThresh = 0
            status = 3
        if o["stopOnResInc"] > 0 and (resSqAll[nit + 1] / resSqAll[nit]).real > o["resIncThresh"]:   # 308-314
            resIncsTotal += 1
            if resIncsTotal >= o["stopOnResInc"]:
                finished, status = True, 4
        if o["stopOnXdifInc"] > 0 and xdiffAll[nit + 1].real > xdiffAll[nit].real:           # 315-326
            if not lastxdifInc:
                xdifIncsTotal += 1
                lastxdifInc = 1
                if xdifIncsTotal >= o["stopOnXdifInc"]:
                    finished, status = True, 5
        else:
            lastxdifInc = 0
        p = res + betaFact * (res_sq_new / res_sq_old) * p                                  # 328
        res_sq_old = res_sq_new
        xold = x
        nit += 1
        if nit >= NitMax:                                                                    # 332-335
            finished, status = True, 0
    n = nit + 1
    return x, resSqAll[:n], mseAll[:n], xnormAll[:n], xdiffAll[:n], stopThresh, status
