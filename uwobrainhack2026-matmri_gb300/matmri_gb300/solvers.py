"""Iterative solvers with the reference signatures, running on the device.

* ``cgne(A, b, x0, NitMax, opt, gam, R, W)``      — iterativeSolvers/cgne.m:1-341
* ``powermethod(A, x0, NitMax, doAtA, xdiffThresh)`` — iterativeSolvers/powermethod.m:1-67
* ``bfista(A, b, R, lam, x0, NitMax, opt)``       — iterativeSolvers/bfista.m:1-246

``A`` is an ``mrSampOp`` / ``functools.partial(mrSampFunc, ...)`` /
``nufftOp`` / ``sampHighOrder`` (see ``sense.resolve_operator``).  Options
are dicts with the reference's field names; a field that is absent takes the
reference default and a field set to ``None`` is MATLAB's ``[]`` (rule off).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .arrays import alloc_like, as_c64, finish, is_torch, stream_of
from .sense import resolve_operator

_NAN = float("nan")


def _d(v):
    return _NAN if v is None else float(v)


def _tik_diag(op, gam, R):
    """sum_k gam_k |R_k|^2 for scalar / elementwise-mask R (cgne.m:171-179, Asub 343-358)."""
    if gam is None:
        return None
    gl = list(gam) if isinstance(gam, (list, tuple)) else [gam]
    Rl = list(R) if isinstance(R, (list, tuple)) else [R]
    if not isinstance(gam, (list, tuple)) and np.all(np.asarray(gam) == 0):
        return None                                                        # cgne.m:91-93
    n = int(np.prod(op.imN))
    acc = np.zeros(n, dtype=np.float64)
    for g, r in zip(gl, Rl):
        if r is None:
            raise ValueError("gam given without R")
        if hasattr(r, "mtimes"):
            raise NotImplementedError("operator-valued Tikhonov R is not supported (use a mask or scalar)")
        ra = np.asarray(r.cpu() if is_torch(r) else r)
        m2 = np.abs(ra.astype(np.complex128)) ** 2
        acc += float(np.real(g)) * (np.broadcast_to(m2.reshape(-1, order="F"), (n,)) if m2.size > 1 else m2.reshape(-1)[0])
    return np.ascontiguousarray(acc.astype(np.float32))


def _scalar_opts(o, NitMax):
    """cgne's scalar options (cgne.m:21-89) in the C struct; absent fields keep the defaults."""
    co = _lib.CgneOpts()
    _lib.check(_lib.load().mmr_cgne_default_opts(C.byref(co)))
    co.nit_max = 1000 if NitMax is None else int(NitMax)
    if "resThresh" in o: co.res_thresh = _d(o["resThresh"])
    if "resChangeThresh" in o: co.res_change_thresh = _d(o["resChangeThresh"])
    if "xChangeThresh" in o: co.x_change_thresh = _d(o["xChangeThresh"])
    if "expResN" in o: co.exp_res_n = int(o["expResN"])
    if "nseThreshFact" in o: co.nse_thresh_fact = float(o["nseThreshFact"])
    if "nseExtraIt" in o: co.nse_extra_it = int(o["nseExtraIt"])
    if "stopOnResInc" in o: co.stop_on_res_inc = int(o["stopOnResInc"])
    if "resIncThresh" in o: co.res_inc_thresh = float(o["resIncThresh"])
    if "stopOnXdifInc" in o: co.stop_on_xdif_inc = int(o["stopOnXdifInc"])
    if "noiseVar" in o: co.noise_var = _d(o["noiseVar"])
    return co


def cgne(A, b, x0=None, NitMax=None, opt=None, gam=None, R=None, W=None):
    """[x, resSqAll, mseAll, xnormAll, xdiffAll, stopThresh, status] = cgne(A, b, x0, NitMax, opt, gam, R, W)."""
    op = resolve_operator(A)
    lib = _lib.load()
    o = dict(opt or {})
    co = _scalar_opts(o, NitMax)
    keep = []
    if o.get("noise") is not None:
        nb = as_c64(o["noise"])
        keep.append(nb)
        co.noise = nb.ptr
    co.noise_seed = int(o.get("noiseSeed", 0))
    if o.get("gtruth") is not None:
        g = as_c64(o["gtruth"])
        keep.append(g)
        co.gtruth = g.ptr
    tik = _tik_diag(op, gam, R)
    if op.tikReg:
        t2 = np.full(int(np.prod(op.imN)), 0.0, dtype=np.float32)
        tik = t2 if tik is None else tik
    if tik is not None:
        co.tik_diag = _lib.fptr(tik)
    Wp = None
    if W is not None:
        w = np.ascontiguousarray(np.asarray(W.cpu() if is_torch(W) else W, dtype=np.float32).reshape(-1, order="F"))
        if w.size not in (op.M, op.M * op.C):
            raise ValueError("W must have M or M*C entries")
        co.w_per_coil = int(w.size == op.M * op.C and op.C > 1)
        keep.append(w)
        Wp = _lib.fptr(w)
    bb = as_c64(b)
    if op.tikReg:
        nda = int(np.prod(op.data_shape))
        if bb.shape[0] > nda if len(bb.shape) == 1 else False:
            tail = np.asarray(b[nda:].cpu() if is_torch(b) else b[nda:])
            if np.any(tail != 0):
                raise NotImplementedError("cgne with opt.tikReg needs the stacked Tikhonov rows of b to be zero")
            bb = as_c64(b[:nda])
    x0b = as_c64(x0) if x0 is not None else None
    out, optr = alloc_like(bb, op.imN)
    cap = co.nit_max + max(co.nse_extra_it, 0) + 1
    hist_arr = np.zeros((4, cap), dtype=np.float64)
    h = _lib.CgneHist()
    h.res_sq = _lib.dptr(hist_arr[0])
    h.mse = _lib.dptr(hist_arr[1])
    h.xnorm = _lib.dptr(hist_arr[2])
    h.xdiff = _lib.dptr(hist_arr[3])
    h.capacity = cap
    _lib.check(lib.mmr_cgne_solve(op.handle, bb.ptr, x0b.ptr if x0b else None, Wp, C.byref(co), optr, C.byref(h),
                                  stream_of(bb)))
    n = h.n
    x = finish(out, bb)
    if op.opt["imNFull"] is not None:
        x = x.permute(*range(x.dim() - 1, -1, -1)).reshape(-1) if is_torch(x) else np.reshape(x, -1, order="F")
    st = None if math.isnan(h.stop_thresh) else h.stop_thresh
    return x, hist_arr[0, :n].copy(), hist_arr[1, :n].copy(), hist_arr[2, :n].copy(), hist_arr[3, :n].copy(), st, h.status


def cgne_batch(As, bs, NitMax=None, opt=None):
    """xs, infos = cgne_batch([A_1..A_n], [b_1..b_n], NitMax, opt): n independent cgne solves (the
    reference loops cgne over slices) advanced together, one CUDA graph launch per iteration for the
    whole batch.  Scalar options as cgne's; x0 = A_i'b_i; infos[i] holds resSqAll, xnormAll, xdiffAll,
    status and nit of solve i."""
    ops = [resolve_operator(A) for A in As]
    n = len(ops)
    if n == 0 or len(bs) != n:
        raise ValueError("cgne_batch needs one data array per operator")
    if len({id(op) for op in ops}) != n:
        raise ValueError("the operators of a batch must be distinct")
    lib = _lib.load()
    co = _scalar_opts(dict(opt or {}), NitMax)
    bufs = [as_c64(b) for b in bs]
    outs = [alloc_like(bb, op.imN) for bb, op in zip(bufs, ops)]
    cap = co.nit_max + max(co.nse_extra_it, 0) + 1
    harr = np.zeros((n, 4, cap), dtype=np.float64)
    hs = (_lib.CgneHist * n)()
    for i in range(n):
        hs[i].res_sq = _lib.dptr(harr[i, 0])
        hs[i].mse = _lib.dptr(harr[i, 1])
        hs[i].xnorm = _lib.dptr(harr[i, 2])
        hs[i].xdiff = _lib.dptr(harr[i, 3])
        hs[i].capacity = cap
    handles = (C.c_void_p * n)(*[op.handle for op in ops])
    bptr = (C.c_void_p * n)(*[bb.ptr for bb in bufs])
    xptr = (C.c_void_p * n)(*[p for _, p in outs])
    _lib.check(lib.mmr_cgne_solve_batch(handles, n, bptr, xptr, C.byref(co), hs, stream_of(bufs[0])))
    xs = [finish(o_, bb) for (o_, _), bb in zip(outs, bufs)]
    infos = [{"resSqAll": harr[i, 0, :hs[i].n].copy(), "xnormAll": harr[i, 2, :hs[i].n].copy(),
              "xdiffAll": harr[i, 3, :hs[i].n].copy(), "status": hs[i].status, "nit": hs[i].nit}
             for i in range(n)]
    return xs, infos


def powermethod(A, x0, NitMax=None, doAtA=None, xdiffThresh=None):
    """maxEig = powermethod(A, x0, NitMax=50, doAtA=1, xdiffThresh=1e-3)."""
    if doAtA is not None and not doAtA:
        raise NotImplementedError("powermethod with doAtA = 0 needs a square operator")
    op = resolve_operator(A)
    lib = _lib.load()
    xb = as_c64(x0)
    re, im = C.c_double(), C.c_double()
    _lib.check(lib.mmr_powermethod(op.handle, xb.ptr, 50 if NitMax is None else int(NitMax),
                                   1e-3 if xdiffThresh is None else float(xdiffThresh), C.byref(re), C.byref(im),
                                   stream_of(xb)))
    return complex(re.value, im.value)


class dwtND:
    """W = dwtND(J, imSize, decimation=False, family='db1') — the undecimated Haar used by bfista.

    Only the configuration the reconstruction path uses is built: db1,
    undecimated (operators/@dwtND/dwtND.m:28-79, filters / sqrt(2) at 111-116).
    """

    def __init__(self, J, imSize, decimation=False, family="db1", useGPUFlag=1):
        if decimation or family != "db1":
            raise NotImplementedError("only the undecimated db1 dwtND is supported")
        imSize = [int(s) for s in imSize]
        J = list(np.broadcast_to(np.asarray(J, dtype=int), (len(imSize),)))
        self.J = [0 if imSize[d] == 1 else int(J[d]) for d in range(len(imSize))]   # dwtND.m:55
        self.imSize = imSize
        self.adjoint = 0

    @property
    def nbands(self):
        n = 1
        for j in range(1, max(self.J) + 1):
            n += 2 ** sum(1 for d in self.J if d >= j) - 1
        return n

    def ctranspose(self):
        o = dwtND.__new__(dwtND)
        o.__dict__.update(self.__dict__)
        o.adjoint = 1 - self.adjoint
        return o

    @property
    def H(self):
        return self.ctranspose()

    def mtimes(self, x):
        """W*x -> list of bands [low, high{1}{1..}, ...]; W'*bands -> image (@dwtND/mtimes.m)."""
        lib = _lib.load()
        nd = len(self.imSize)
        imN = (C.c_int64 * 3)(*(self.imSize + [1] * (3 - nd)))
        lev = (C.c_int32 * 3)(*(self.J + [0] * (3 - nd)))
        nb = self.nbands
        if not self.adjoint:
            b = as_c64(x)
            out, optr = alloc_like(b, list(self.imSize) + [nb])
            _lib.check(lib.mmr_dwt_haar(nd, imN, lev, 0, b.ptr, optr, stream_of(b)))
            out = finish(out, b)
            return [out[..., k] for k in range(nb)]
        bands = x
        if is_torch(bands[0]):
            import torch
            stacked = torch.stack(list(bands), dim=-1)
        else:
            stacked = np.stack(list(bands), axis=-1)
        b = as_c64(stacked)
        out, optr = alloc_like(b, self.imSize)
        _lib.check(lib.mmr_dwt_haar(nd, imN, lev, 1, b.ptr, optr, stream_of(b)))
        return finish(out, b)

    __mul__ = lambda self, x: self.mtimes(x)


def bfista(A, b, R, lam, x0=None, NitMax=None, opt=None):
    """[x, resSqAll, RxAll, testAll, maxEig] = bfista(A, b, R, lam, x0, NitMax, opt)."""
    op = resolve_operator(A)
    if not isinstance(R, dwtND):
        raise TypeError("R must be a dwtND (undecimated db1)")
    lib = _lib.load()
    o = dict(opt or {})
    nit = 200 if NitMax is None else int(NitMax)
    bo = _lib.BfistaOpts()
    bo.nit_max = nit
    bo.res_thresh = float(o.get("resThresh", 1e-5))
    me = o.get("maxEig")
    bo.max_eig = -1.0 if me is None else float(abs(me))
    bo.n_restart = int(o.get("nRestart", nit + 1))
    keep = []
    if o.get("xMask") is not None:
        xm = as_c64(o["xMask"])
        keep.append(xm)
        bo.x_mask = xm.ptr
    nb = R.nbands
    lam_a = np.ascontiguousarray(np.broadcast_to(np.asarray(lam, dtype=np.float32).reshape(-1), (nb,)).copy()
                                 if np.size(lam) in (1, nb) else None)
    if lam_a is None:
        raise ValueError(f"lam must be a scalar or have {nb} per-band entries")
    lev = (C.c_int32 * 3)(*(list(R.J) + [0] * (3 - len(R.J))))
    bb = as_c64(b)
    x0b = as_c64(x0) if x0 is not None else None
    out, optr = alloc_like(bb, op.imN)
    hist = np.zeros((4, nit), dtype=np.float64)
    h = _lib.BfistaHist()
    h.res_sq = _lib.dptr(hist[0])
    h.rx = _lib.dptr(hist[1])
    test = np.zeros(2 * nit, dtype=np.float64)
    h.test = _lib.dptr(test)
    h.capacity = nit
    _lib.check(lib.mmr_bfista_solve(op.handle, bb.ptr, lev, _lib.fptr(lam_a), nb, x0b.ptr if x0b else None,
                                    C.byref(bo), optr, C.byref(h), stream_of(bb)))
    n = h.n
    testAll = test.reshape(nit, 2, order="F")[:n].copy()
    if n:
        testAll[0, :] = np.nan
    return finish(out, bb), hist[0, :n].copy(), hist[1, :n].copy(), testAll, h.max_eig
