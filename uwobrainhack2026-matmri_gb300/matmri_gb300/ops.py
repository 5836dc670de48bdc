"""Drop-in operator classes: ``nufftOp``, ``rcvrOp``, ``sampHighOrder``.

Constructor arguments, defaults and the ``N*x`` / ``N'*y`` semantics follow
the reference classes:
  * nufftOp       — operators/@nufftOp/nufftOp.m:89-136 (ctor), 276-282
                    (ctranspose/transpose), 284-408 (mtimes), 410-432 (prepToep)
  * rcvrOp        — operators/@rcvrOp/rcvrOp.m:47-94, 96-159
  * sampHighOrder — operators/@sampHighOrder/sampHighOrder.m:129-312

MATLAB's ``N'`` is ``N.ctranspose()`` or ``N.H``; ``N*x`` is ``N * x``
(also ``N @ x`` and ``N.mtimes(x)``).  Like the value classes of the
reference, ``N.H`` returns a copy with the adjoint flag flipped; copies share
one device plan (a refcounted handle), as a MATLAB handle member would.
Everything runs in the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import copy
import math

import numpy as np

from . import _lib
from .arrays import Buf, alloc_like, as_c64, f64, finish, stream_of


class _Handle:
    """Owns one C handle and destroys it when the last Python reference goes."""

    def __init__(self, ptr, destroy):
        self.ptr = ptr
        self._destroy = destroy

    def __del__(self):
        try:
            if self.ptr:
                self._destroy(self.ptr)
        except Exception:
            pass
        self.ptr = None


class _Op:
    adjoint = 0

    def ctranspose(self):
        o = copy.copy(self)
        o.adjoint = 1 - self.adjoint
        return o

    def transpose(self):
        return self.ctranspose()

    @property
    def H(self):
        return self.ctranspose()

    def __mul__(self, x):
        return self.mtimes(x)

    def __matmul__(self, x):
        return self.mtimes(x)


class nufftOp(_Op):
    """N = nufftOp(imN, kloc, dcf=[], useGPU=1, os=1.5, kwidth=6)."""

    def __init__(self, imN=None, kloc=None, dcf=None, useGPU=None, os=None, kwidth=None):
        if imN is None:
            raise TypeError("nufftOp() with no arguments runs the reference self-tests; use pytest tests/")
        lib = _lib.load()
        self.imgN = [int(n) for n in np.atleast_1d(imN)]
        nd = len(self.imgN)
        k = np.asarray(kloc, dtype=np.float64)
        if k.ndim == 1:
            k = k.reshape(-1, 1)
        if k.shape[1] != nd:
            raise ValueError(f"kloc must be [M x {nd}]")
        self.kloc = np.asfortranarray(k)
        self.os = 1.5 if os is None else float(os)             # nufftOp.m:66
        self.kwidth = 6 if kwidth is None else int(kwidth)     # nufftOp.m:65
        self.useGPU = 1
        self.useSingle = 0
        self.loopDim = 4
        self.isToep = False
        d = _lib.NufftDesc()
        d.ndim = nd
        for i in range(3):
            d.imN[i] = self.imgN[i] if i < nd else 1
        d.nsamp = self.kloc.shape[0]
        d.kloc = _lib.dptr(self.kloc)
        dc = None if dcf is None or np.size(dcf) == 0 else f64(dcf, d.nsamp)
        d.dcf = _lib.dptr(dc) if dc is not None else None
        d.os = self.os
        d.kwidth = self.kwidth
        h = C.c_void_p()
        _lib.check(lib.mmr_nufft_create(C.byref(d), C.byref(h)))
        self._h = _Handle(h.value, lib.mmr_nufft_destroy)
        self._dcf = dc
        osN = (C.c_int64 * 3)()
        beta = C.c_double()
        nk = C.c_int64()
        _lib.check(lib.mmr_nufft_info(self._h.ptr, osN, C.byref(beta), C.byref(nk)))
        self.osN = [int(osN[i]) for i in range(nd)]
        self.beta = beta.value
        self.Nkern = nk.value

    @property
    def dcf(self):
        return self._dcf

    @dcf.setter
    def dcf(self, v):
        """``Nop.dcf = dcf`` (demos/demo_regridding.m:35, 45)."""
        lib = _lib.load()
        if v is None or np.size(v) == 0:
            self._dcf = None
            _lib.check(lib.mmr_nufft_set_dcf(self._h.ptr, None))
        else:
            self._dcf = f64(v, self.kloc.shape[0])
            _lib.check(lib.mmr_nufft_set_dcf(self._h.ptr, _lib.dptr(self._dcf)))

    @property
    def handle(self):
        return self._h.ptr

    def mtimes(self, x):
        lib = _lib.load()
        nd = len(self.imgN)
        b = as_c64(x)
        shp = list(b.shape)
        M = self.kloc.shape[0]
        if self.isToep or not self.adjoint:
            if shp[:nd] != self.imgN:
                raise ValueError(f"input must be [{self.imgN}, extra...], got {shp}")
            extra = shp[nd:]
            out_shape = (self.imgN if self.isToep else [M]) + extra
        else:
            if shp[0] != M:
                raise ValueError(f"input must be [{M}, extra...], got {shp}")
            extra = shp[1:]
            out_shape = self.imgN + extra
        nb = int(np.prod(extra)) if extra else 1
        out, optr = alloc_like(b, out_shape)
        _lib.check(lib.mmr_nufft_apply(self._h.ptr, int(self.adjoint), b.ptr, optr, nb, stream_of(b)))
        return finish(out, b)

    def prepToep(self, tos=None, kwidth=None):
        """S = S.prepToep(tos, kwidth): returns a Toeplitz copy (nufftOp.m:410-432)."""
        if self.isToep:
            return self
        o = nufftOp(self.imgN, self.kloc, self._dcf, 1, self.os, self.kwidth)
        _lib.check(_lib.load().mmr_nufft_prep_toep(o._h.ptr, -1.0 if tos is None else float(tos),
                                                   -1 if kwidth is None else int(kwidth)))
        o.isToep = True
        o.loopDim = self.loopDim + 1
        return o

    def findDcf(self, nit=None, isIt=False):
        raise NotImplementedError("nufftOp.findDcf (lsqlin-based DCF, nufftOp.m:434-477) is not supported")


class rcvrOp(_Op):
    """R = rcvrOp(maps, isCalDat=0): coil sensitivities, last dim = receivers."""

    def __init__(self, input=None, isCalDat=0, apN=None, kalph=None):
        if input is None:
            raise TypeError("rcvrOp() with no arguments runs the reference self-tests; use pytest tests/")
        if isCalDat:
            raise NotImplementedError("rcvrOp calibration from low-res data (rcvrOp.m:66-89) is a set-up step "
                                      "not supported; pass precomputed maps with isCalDat = 0")
        lib = _lib.load()
        m = np.asfortranarray(np.asarray(input), dtype=np.complex64)
        self.maps = m
        self.imgN = list(m.shape)
        self.nDim = m.ndim - 1
        self.doLoop = 0
        imN = (C.c_int64 * 3)(*([int(s) for s in m.shape[:-1]] + [1] * (4 - m.ndim)))
        h = C.c_void_p()
        _lib.check(lib.mmr_rcvr_create(self.nDim, imN, int(m.shape[-1]), m.ctypes.data, C.byref(h)))
        self._h = _Handle(h.value, lib.mmr_rcvr_destroy)

    @property
    def handle(self):
        return self._h.ptr

    def mtimes(self, x):
        lib = _lib.load()
        b = as_c64(x)
        N = self.imgN[:-1]
        out_shape = N if self.adjoint else self.imgN
        out, optr = alloc_like(b, out_shape)
        _lib.check(lib.mmr_rcvr_apply(self._h.ptr, int(self.adjoint), b.ptr, optr, stream_of(b)))
        return finish(out, b)


class sampHighOrder(_Op):
    """S = sampHighOrder(b0, sampTimes, phs_spha, phs_conc, phs_grid, imMask, useGPU, useSingle, approach, opt).

    Approaches 0, 2 and 3 compute the same sums (direct / segmented) and map
    to the same device kernels.  Approach 1 is the SVD + NUFFT interpolated
    encoding (sampHighOrder.m:314-359, prepForInterp 700-889): the factors
    are formed on the host (``sho_interp.prep_for_interp``; opt.svdThresh,
    opt.subFact, opt.svdNtry) and applied on the device; opt.subFactSpc > 1
    and SMS slice stacks are not supported (ValueError).  The factors stay
    readable as ``svdSpace``, ``svdTime``, ``phsShft`` and the trajectory
    ``traj_kloc``.
    """

    def __init__(self, b0=None, sampTimes=None, phs_spha=None, phs_conc=None, phs_grid=None, b0mask=None,
                 useGPU=None, useSingle=None, approach=None, opt=None):
        if sampTimes is None:
            raise TypeError("sampHighOrder() with no arguments runs the reference self-tests; use pytest tests/")
        self.approach = 0 if approach is None else int(approach)
        if self.approach == 1:
            self._init_interp(b0, sampTimes, phs_spha, phs_conc, phs_grid, b0mask, opt or {})
            return
        lib = _lib.load()
        gx = np.asarray(phs_grid["x"], dtype=np.float64)
        self.imSize = list(gx.shape) if not (gx.ndim == 2 and gx.shape[1] == 1) else [gx.shape[0]]
        t = np.asarray(sampTimes, dtype=np.float64)
        self.kSize = list(t.shape) if not (t.ndim == 2 and t.shape[1] == 1) else [t.shape[0]]
        V = gx.size
        M = t.size
        sp = np.asarray(phs_spha, dtype=np.float64).reshape(np.shape(phs_spha)[0], -1, order="F")
        if sp.shape[1] != M:
            raise ValueError("Dimension mismatch between phs_spha and sampTimes")   # sampHighOrder.m:243-245
        pc = np.zeros((0, M)) if phs_conc is None or np.size(phs_conc) == 0 else \
            np.asarray(phs_conc, dtype=np.float64).reshape(np.shape(phs_conc)[0], -1, order="F")
        if b0 is not None and np.size(b0) and np.size(b0) != V:
            raise ValueError("Size mismatch between b0 and phs_grid.x")                # sampHighOrder.m:223-224
        self._keep = dict(
            b0=f64(b0) if b0 is not None and np.size(b0) else None,
            t=f64(t), spha=np.asfortranarray(sp), conc=np.asfortranarray(pc),
            gx=f64(gx), gy=f64(phs_grid["y"]), gz=f64(phs_grid["z"]),
            mask=f64(b0mask) if b0mask is not None and np.size(b0mask) else None)
        k = self._keep
        d = _lib.ShoDesc()
        d.ndim = len(self.imSize)
        for i in range(3):
            d.imN[i] = self.imSize[i] if i < len(self.imSize) else 1
        d.nsamp = M
        d.nspha = sp.shape[0]
        d.nconc = pc.shape[0]
        d.b0 = _lib.dptr(k["b0"]) if k["b0"] is not None else None
        d.t = _lib.dptr(k["t"])
        d.spha = _lib.dptr(k["spha"])
        d.conc = _lib.dptr(k["conc"]) if pc.shape[0] else None
        d.gx, d.gy, d.gz = _lib.dptr(k["gx"]), _lib.dptr(k["gy"]), _lib.dptr(k["gz"])
        d.mask = _lib.dptr(k["mask"]) if k["mask"] is not None else None
        h = C.c_void_p()
        _lib.check(lib.mmr_sho_create(C.byref(d), C.byref(h)))
        self._h = _Handle(h.value, lib.mmr_sho_destroy)
        self.V, self.M = V, M

    def _init_interp(self, b0, sampTimes, phs_spha, phs_conc, phs_grid, b0mask, opt):
        from .sho_interp import prep_for_interp
        opt = dict(opt)
        if opt.get("subFactSpc") not in (None, 1):
            raise ValueError("opt.subFactSpc > 1 is not supported by the interpolated approach here")
        lib = _lib.load()
        gx = np.asarray(phs_grid["x"], dtype=np.float64)
        if gx.ndim != 2:
            raise ValueError("the interpolated approach is built for 2-D grids (no SMS slice stacks)")
        t = np.asarray(sampTimes, dtype=np.float64)
        self._t = t
        self.imSize = list(gx.shape)
        self.kSize = list(t.shape) if not (t.ndim == 2 and t.shape[1] == 1) else [t.shape[0]]
        if b0 is not None and np.size(b0) and np.size(b0) != gx.size:
            raise ValueError("Size mismatch between b0 and phs_grid.x")                # sampHighOrder.m:223-224
        self.svdThresh = 0.05 if opt.get("svdThresh") is None else float(opt["svdThresh"])
        self.subFact = 5 if opt.get("subFact") is None else max(1, int(opt["subFact"]))
        f = prep_for_interp(b0, t, phs_spha, phs_conc, phs_grid, b0mask, self.svdThresh, self.subFact,
                            opt.get("svdNtry"))
        self.svdSpace, self.svdTime, self.phsShft, self.traj_kloc = f["svdSpace"], f["svdTime"], f["phsShft"], \
            f["kloc"]
        L = f["s"].size
        k = dict(kloc=np.asfortranarray(f["kloc"]),
                 space=np.asfortranarray(f["svdSpace"], dtype=np.complex128),
                 time=np.asfortranarray(f["svdTime"], dtype=np.complex128),
                 shift=np.ascontiguousarray(f["phsShft"], dtype=np.complex128))
        self._keep = k
        d = _lib.ShoInterpDesc()
        d.ndim = 2
        d.imN[0], d.imN[1], d.imN[2] = self.imSize[0], self.imSize[1], 1
        d.nsamp = t.size
        d.nterms = L
        cp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        d.kloc, d.svd_space, d.svd_time, d.phs_shift = cp(k["kloc"]), cp(k["space"]), cp(k["time"]), cp(k["shift"])
        d.os, d.kwidth = 0.0, 0
        h = C.c_void_p()
        _lib.check(lib.mmr_sho_interp_create(C.byref(d), C.byref(h)))
        self._h = _Handle(h.value, lib.mmr_sho_destroy)
        self.V, self.M = gx.size, t.size

    def setPhiDiv(self, ksphaDiv, kconcDiv):
        """S2 = S.setPhiDiv(ksphaDiv, kconcDiv) (sampHighOrder.m:590-622), a copy (value semantics).

        The copy's forward is (1i * exp(1i*kbase) .* phiDiv).' * x / sqrt(V)
        (useDirectWorker, 374-381); its adjoint ignores phiDiv (369-372).
        For the interpolated approach the forward raises, as the reference's
        useInterpWorker does (340-342).
        """
        o = copy.copy(self)
        o._phidiv_base = self
        if self.approach == 1:
            o._phidiv_unsupported = True
            return o
        ks = np.asarray(ksphaDiv, dtype=np.float64)
        ks = np.zeros((0, self.M)) if ks.size == 0 else ks.reshape(ks.shape[0], -1, order="F")
        kc = np.asarray(kconcDiv, dtype=np.float64) if kconcDiv is not None else np.zeros((0, self.M))
        kc = np.zeros((0, self.M)) if kc.size == 0 else kc.reshape(kc.shape[0], -1, order="F")
        if ks.shape[1] != self.M or kc.shape[1] != self.M:
            raise ValueError("Dimension mismatch between phiDiv and sampTimes")
        ks, kc = np.asfortranarray(ks), np.asfortranarray(kc)
        o._keep_phidiv = (ks, kc)
        lib = _lib.load()
        h = C.c_void_p()
        cp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double)) if a.size else None
        _lib.check(lib.mmr_sho_phidiv_create(self.handle, ks.shape[0], kc.shape[0], cp(ks), cp(kc), C.byref(h)))
        o._h = _Handle(h.value, lib.mmr_sho_destroy)
        return o

    def updateObj(self, phs_spha, phs_conc, b0map, b0mask, phs_grid):
        """sampHighOrder.m:889-934: rebuilds the interpolated plan for new inputs (approach 1 only)."""
        if self.approach != 1:
            raise ValueError("this case not yet coded")                            # sampHighOrder.m:932
        opt = {"svdThresh": self.svdThresh, "subFact": self.subFact}
        o = copy.copy(self)
        o._init_interp(b0map, self._t, phs_spha, phs_conc, phs_grid, b0mask, opt)
        return o

    def set_tensor(self, mode=1):
        """Contraction of the direct encoding: 1 / True the tcgen05 tensor-core kernel (default),
        2 the mma.sync tensor-core kernel, 0 / False the SIMT FP32 kernels."""
        _lib.check(_lib.load().mmr_sho_set_tensor(self.handle, int(mode)))
        return self

    @property
    def kbase(self):
        """The FP64 encoding phase [V x M] of a direct plan (prepForDirect, sampHighOrder.m:496-588; the
        matrix operators/mrSampFuncMat.m:35 reads), evaluated on the device from the plan's basis."""
        if self.approach == 1:
            raise AttributeError("kbase is not formed by the interpolated approach")
        out = np.empty((self.V, self.M), dtype=np.float64, order="F")
        _lib.check(_lib.load().mmr_sho_kbase(self.handle, out.ctypes.data))
        return out

    @property
    def handle(self):
        return self._h.ptr

    def mtimes(self, x):
        if getattr(self, "_phidiv_unsupported", False) and not self.adjoint:
            raise ValueError("phiDiv not yet implemented for interpolated approach")   # sampHighOrder.m:340-342
        lib = _lib.load()
        b = as_c64(x)
        shp = list(b.shape)
        if self.adjoint:
            nk = len(self.kSize)
            extra = shp[nk:] if shp[:nk] == self.kSize else shp[1:]
            out_shape = self.imSize + extra
        else:
            ni = len(self.imSize)
            extra = shp[ni:] if shp[:ni] == self.imSize else shp[1:]
            out_shape = self.kSize + extra
        nb = int(np.prod(extra)) if extra else 1
        out, optr = alloc_like(b, out_shape)
        _lib.check(lib.mmr_sho_apply(self._h.ptr, int(self.adjoint), b.ptr, optr, nb, stream_of(b)))
        return finish(out, b)
