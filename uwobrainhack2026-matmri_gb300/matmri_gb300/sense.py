"""``mrSampFunc`` — the SENSE encoding function handle (operators/mrSampFunc.m).

``mrSampFunc(x, transp, samplingOp, R, opt)`` has the reference signature.
MATLAB scripts build ``opFunc = @(x,transp) mrSampFunc(x,transp,S,R,opt)``;
the Python equivalents are ``mrSampOp(S, R, opt)`` (a callable object) or
``functools.partial(mrSampFunc, samplingOp=S, R=R, opt=opt)`` — both are
recognised by ``cgne`` / ``bfista`` / ``powermethod``, which then run the
whole solve on the device.
"""
from __future__ import annotations

import ctypes as C
import functools

import numpy as np

from . import _lib
from .arrays import alloc_like, as_c64, finish, is_torch, stream_of
from .ops import _Handle, nufftOp, rcvrOp, sampHighOrder


def _opt(opt):
    o = dict(opt or {})
    for k in ("imNFull", "daNFull", "tikReg", "sumDims", "hardReal", "W"):
        o.setdefault(k, None)
    return o


class mrSampOp:
    """Callable ``A(x, transp)`` equal to ``mrSampFunc(x, transp, S, R, opt)``."""

    def __init__(self, samplingOp, R=None, opt=None):
        if not isinstance(samplingOp, (nufftOp, sampHighOrder)):
            raise NotImplementedError("mrSampFunc with a Cartesian mask sampling operator (mrSampFunc.m:109-113) "
                                      "is not supported; use nufftOp or sampHighOrder")
        if R is not None and not isinstance(R, rcvrOp):
            raise TypeError("R must be an rcvrOp")
        if isinstance(samplingOp, nufftOp) and samplingOp.isToep:
            raise ValueError("a Toeplitz nufftOp cannot be used inside mrSampFunc")
        o = _opt(opt)
        if o["sumDims"]:
            raise NotImplementedError("opt.sumDims is not supported")
        tr = o["tikReg"]
        if tr is not None and np.size(tr) != 1:
            raise NotImplementedError("a two-element opt.tikReg is not supported")
        if tr is not None and (o["imNFull"] is None or o["daNFull"] is None):
            raise ValueError("Tikhonov regularization requires opt.imNFull and opt.daNFull")   # mrSampFunc.m:78-80
        self.S, self.R, self.opt = samplingOp, R, o
        self.tikReg = 0.0 if tr is None else float(np.asarray(tr).reshape(-1)[0])
        lib = _lib.load()
        d = _lib.SenseDesc()
        if isinstance(samplingOp, nufftOp):
            d.nufft = samplingOp.handle
            self.imN = list(samplingOp.imgN)
            self.M = samplingOp.kloc.shape[0]
            self.kshape = [self.M]
        else:
            d.sho = samplingOp.handle
            self.imN = list(samplingOp.imSize)
            self.M = samplingOp.M
            self.kshape = list(samplingOp.kSize)
        d.rcvr = R.handle if R is not None else None
        self.C = R.imgN[-1] if R is not None else 1
        self._W = None
        if o["W"] is not None:
            w = np.asarray(o["W"], dtype=np.float32).reshape(-1, order="F")
            if w.size not in (self.M, self.M * self.C):
                raise ValueError("opt.W must have M or M*C entries")
            self._W = np.ascontiguousarray(w)
            d.W = _lib.fptr(self._W)
            d.w_per_coil = int(w.size == self.M * self.C and self.C > 1)
        d.tikreg = self.tikReg
        h = C.c_void_p()
        _lib.check(lib.mmr_sense_create(C.byref(d), C.byref(h)))
        self._h = _Handle(h.value, lib.mmr_sense_destroy)

    @property
    def handle(self):
        return self._h.ptr

    @property
    def data_shape(self):
        return self.kshape + ([self.C] if self.R is not None else [])

    def set_tuning(self, coil_chunk=0, tile=0, coil_group=0, item=0, fft_lines=0, normal_mode=0):
        """Sets the autotuner knobs (0 keeps the current value); see mmr_tuning."""
        t = _lib.Tuning(int(coil_chunk), int(tile), int(coil_group), int(item), int(fft_lines), int(normal_mode))
        _lib.check(_lib.load().mmr_sense_set_tuning(self.handle, C.byref(t)))

    def get_tuning(self):
        """(coil_chunk, tile, coil_group, item, fft_lines, normal_mode)."""
        t = _lib.Tuning()
        _lib.check(_lib.load().mmr_sense_get_tuning(self.handle, C.byref(t)))
        return t.coil_chunk, t.tile, t.coil_group, t.item, t.fft_lines, t.normal_mode

    def __call__(self, x, transp):
        lib = _lib.load()
        o = self.opt
        if transp == "notransp":                                           # mrSampFunc.m:83-120
            if o["hardReal"]:
                x = x.real if is_torch(x) else np.real(x)
            x_tik = None
            if self.tikReg:
                x_tik = self.tikReg * x
            b = as_c64(x if o["imNFull"] is None else _reshape(x, self.imN))
            out, optr = alloc_like(b, self.data_shape)
            _lib.check(lib.mmr_sense_apply(self.handle, 0, b.ptr, optr, stream_of(b)))
            y = finish(out, b)
            if o["daNFull"] is not None:
                y = _vec(y)
            if x_tik is not None:
                y = _cat(y, _vec(x_tik))
            return y
        if transp != "transp":
            raise ValueError("transp must be 'notransp' or 'transp'")
        x_tik = None
        if self.tikReg:                                                    # 122-125
            nda = int(np.prod(o["daNFull"]))
            x, x_tik = x[:nda], x[nda:]
        b = as_c64(x if o["daNFull"] is None else _reshape(x, self.data_shape))
        out, optr = alloc_like(b, self.imN)
        _lib.check(lib.mmr_sense_apply(self.handle, 1, b.ptr, optr, stream_of(b)))
        y = finish(out, b)
        if o["imNFull"] is not None:
            y = _vec(y)
        if x_tik is not None:
            y = y + self.tikReg * x_tik
        if o["hardReal"]:
            y = y.real if is_torch(y) else np.real(y)
        return y

    def normal(self, x):
        """A'(A x) with the fused gridding (one call, no k-space round trip)."""
        lib = _lib.load()
        b = as_c64(x)
        out, optr = alloc_like(b, b.shape)
        _lib.check(lib.mmr_sense_normal(self.handle, b.ptr, optr, stream_of(b)))
        return finish(out, b)


def _reshape(x, shape):
    if is_torch(x):
        return x.reshape(list(shape)[::-1]).permute(*range(len(shape) - 1, -1, -1))
    return np.reshape(x, shape, order="F")


def _vec(x):
    if is_torch(x):
        return x.permute(*range(x.dim() - 1, -1, -1)).reshape(-1)
    return np.reshape(x, -1, order="F")


def _cat(a, b):
    if is_torch(a):
        import torch
        return torch.cat([a, b])
    return np.concatenate([a, b])


_CACHE: dict = {}


def _key(samplingOp, R, opt):
    o = _opt(opt)
    w = o["W"]
    return (id(samplingOp), samplingOp.handle, id(R), R.handle if R is not None else None,
            id(w) if w is not None else None, repr(o["tikReg"]), repr(o["imNFull"]), repr(o["daNFull"]),
            repr(o["hardReal"]), repr(o["sumDims"]))


def get_op(samplingOp, R=None, opt=None) -> mrSampOp:
    k = _key(samplingOp, R, opt)
    op = _CACHE.get(k)
    if op is None or op.S is not samplingOp or op.R is not R:
        if len(_CACHE) > 32:
            _CACHE.clear()
        op = mrSampOp(samplingOp, R, opt)
        _CACHE[k] = op
    return op


def mrSampFunc(x=None, transp=None, samplingOp=None, R=None, opt=None):
    """y = mrSampFunc(x, transp, samplingOp, R, opt)  (operators/mrSampFunc.m:1-160)."""
    if x is None:
        raise TypeError("mrSampFunc() with no arguments runs the reference self-tests; use pytest tests/")
    return get_op(samplingOp, R, opt)(x, transp)


def resolve_operator(A) -> mrSampOp:
    """Maps the A accepted by cgne/bfista/powermethod to a native mrSampOp."""
    if isinstance(A, mrSampOp):
        return A
    if isinstance(A, (nufftOp, sampHighOrder)):
        if A.adjoint:
            raise NotImplementedError("solving with an adjoint operator is not supported")
        return get_op(A, None, None)
    if isinstance(A, functools.partial) and A.func is mrSampFunc:
        kw = dict(A.keywords)
        args = list(A.args)
        S = kw.pop("samplingOp", args[2] if len(args) > 2 else None)
        R = kw.pop("R", args[3] if len(args) > 3 else None)
        opt = kw.pop("opt", args[4] if len(args) > 4 else None)
        return get_op(S, R, opt)
    raise TypeError("A must be an mrSampOp, a nufftOp / sampHighOrder, or functools.partial(mrSampFunc, ...): "
                    "arbitrary Python callables cannot run on the device")
