"""Learned preconditioner and warm start for CG-SENSE (no counterpart in the reference).

* ``PrecondNet``  — the bias-free 3x3 CNN of ``include/matmri_gb300.h``
  (``mmr_cnn_*``): forward (BF16 activations, tensor-core hidden layers),
  loss + gradient and Adam steps, all on the device.
* ``lpcg``        — flexible CG on the system ``cgne`` solves, with the network
  as preconditioner (``mmr_lpcg_solve``); ``net=None`` gives plain CG.
* ``make_pairs`` / ``train`` — training pairs from plain-CG solves
  (residual r_k -> error x* - x_k, which is what a preconditioner should
  return) and the training loop over random crops.

Images follow the package convention: column-major complex64, ``x[i1, i2]``;
CUDA torch tensors are used in place, numpy arrays are staged.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .arrays import alloc_like, as_c64, finish, is_torch, stream_of
from .sense import resolve_operator

CHANNELS = (2, 32, 32, 32, 32, 32, 2)


def init_params(seed: int, channels=CHANNELS) -> np.ndarray:
    """He-normal weights (std sqrt(2 / (9 cin))) drawn from numpy PCG64(seed); skip = 0."""
    g = np.random.Generator(np.random.PCG64(seed))
    parts = [g.standard_normal(channels[l + 1] * channels[l] * 9) * math.sqrt(2.0 / (9 * channels[l]))
             for l in range(len(channels) - 1)]
    parts.append(np.zeros(1))
    return np.concatenate(parts).astype(np.float32)


class PrecondNet:
    """z = net(r) on complex images; parameters FP32 (``theta``), activations BF16.

    ``linear=True`` (the default) uses identity activations: the network is then a fixed linear
    operator, which keeps flexible CG as effective as preconditioned CG.  With ReLU activations the
    preconditioner changes with every residual and the solve stalls far above the target accuracy.
    """

    def __init__(self, params=None, seed: int = 0, channels=CHANNELS, linear: bool = True):
        lib = _lib.load()
        ch = (C.c_int32 * len(channels))(*channels)
        h = C.c_void_p()
        _lib.check(lib.mmr_cnn_create(len(channels) - 1, ch, C.byref(h)))
        self._h = h
        self.channels = tuple(channels)
        self.linear = bool(linear)
        self.base_flags = _lib.CNN_LINEAR if self.linear else 0
        n = C.c_int64()
        _lib.check(lib.mmr_cnn_num_params(h, C.byref(n)))
        self.n_params = int(n.value)
        self.set_params(init_params(seed, channels) if params is None else params)

    @property
    def handle(self):
        return self._h

    def set_params(self, theta):
        t = np.ascontiguousarray(np.asarray(theta, dtype=np.float32).reshape(-1))
        if t.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {t.size}")
        _lib.check(_lib.load().mmr_cnn_set_params(self._h, t.ctypes.data))

    def get_params(self) -> np.ndarray:
        t = np.empty(self.n_params, dtype=np.float32)
        _lib.check(_lib.load().mmr_cnn_get_params(self._h, t.ctypes.data))
        return t

    def save(self, path, **meta):
        np.savez(path, theta=self.get_params(), channels=np.array(self.channels), linear=self.linear,
                 **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path):
        f = np.load(path)
        return cls(params=f["theta"], channels=tuple(int(c) for c in f["channels"]), linear=bool(f["linear"]))

    def forward(self, r, flags: int = _lib.CNN_TENSOR):
        """z = net(r) for r [nx, ny] or [nx, ny, batch]."""
        b = as_c64(r)
        shp = tuple(b.shape) + (1,) * (3 - len(b.shape))
        out, optr = alloc_like(b, b.shape)
        _lib.check(_lib.load().mmr_cnn_forward(self._h, b.ptr, optr, shp[0], shp[1], shp[2],
                                               flags | self.base_flags, stream_of(b)))
        return finish(out, b)

    __call__ = forward

    def loss_grad(self, r, e, margin: int = 6, flags: int = 0, want_grad: bool = True):
        """(loss, grad) of one batch r, e [nx, ny, batch]; grad is None unless want_grad."""
        rb, eb = as_c64(r), as_c64(e)
        if tuple(rb.shape) != tuple(eb.shape):
            raise ValueError("r and e must have the same shape")
        shp = tuple(rb.shape) + (1,) * (3 - len(rb.shape))
        L = C.c_double()
        g = np.empty(self.n_params, dtype=np.float32) if want_grad else None
        _lib.check(_lib.load().mmr_cnn_loss_grad(self._h, rb.ptr, eb.ptr, shp[0], shp[1], shp[2], margin,
                                                 flags | self.base_flags, C.byref(L),
                                                 g.ctypes.data if want_grad else None, stream_of(rb)))
        return L.value, g

    def adam_step(self, lr: float, stream=None):
        _lib.check(_lib.load().mmr_cnn_adam_step(self._h, float(lr), stream))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.mmr_cnn_destroy(h)
            self._h = None


def lpcg(A, y, net: PrecondNet | None = None, x0=None, NitMax: int = 100, tol: float = 0.0, lam: float = 0.0,
         tik_diag=None, gtruth=None, stall_window: int = 10, flags: int = _lib.CNN_TENSOR, poll: int = 8,
         fcg_m: int = 4, fold: bool = True):
    """x, res_sq, err_sq, info = lpcg(A, y, net, ...): learned-preconditioned CG-SENSE.

    Solves (A'A + lam + diag(tik_diag)) x = A'y like ``cgne(A, y, x0, NitMax, opt, gam, R)`` with
    gam = lam and R = 1; ``net=None`` runs plain CG in the same kernels.
    """
    op = resolve_operator(A)
    lib = _lib.load()
    o = _lib.LpcgOpts()
    _lib.check(lib.mmr_lpcg_default_opts(C.byref(o)))
    o.nit_max = int(NitMax)
    o.tol = float(tol)
    o.lam = float(lam)
    o.stall_window = int(stall_window)
    # a linear network is applied as its folded filter unless the caller picks the layered path
    folded = _lib.CNN_FOLDED if (net is not None and net.linear and fold) else 0
    o.flags = int(flags) | (net.base_flags if net is not None else 0) | folded
    o.poll = int(poll)
    o.fcg_m = int(fcg_m)
    keep = []
    if tik_diag is not None:
        t = np.ascontiguousarray(np.asarray(tik_diag.cpu() if is_torch(tik_diag) else tik_diag,
                                            dtype=np.float32).reshape(-1, order="F"))
        keep.append(t)
        o.tik_diag = _lib.fptr(t)
    if gtruth is not None:
        g = as_c64(gtruth)
        keep.append(g)
        o.gtruth = g.ptr
    yb = as_c64(y)
    x0b = as_c64(x0) if x0 is not None else None
    out, optr = alloc_like(yb, op.imN)
    cap = o.nit_max + 1
    hist = np.zeros((2, cap), dtype=np.float64)
    h = _lib.LpcgHist()
    h.res_sq = _lib.dptr(hist[0])
    h.err_sq = _lib.dptr(hist[1])
    h.capacity = cap
    _lib.check(lib.mmr_lpcg_solve(op.handle, yb.ptr, net.handle if net is not None else None,
                                  x0b.ptr if x0b else None, C.byref(o), optr, C.byref(h), stream_of(yb)))
    info = {"nit": h.nit, "status": h.status, "fell_back_at": h.fell_back_at, "true_res_rel": h.true_res_rel}
    return finish(out, yb), hist[0, :h.n].copy(), hist[1, :h.n].copy(), info


def iterations_to(err_sq, gnorm: float, target: float = 1e-3):
    """First iteration k with sqrt(err_sq[k]) / gnorm <= target (None if never)."""
    e = np.sqrt(np.asarray(err_sq)) / gnorm
    idx = np.nonzero(e <= target)[0]
    return int(idx[0]) if idx.size else None


# ------------------------------------------------------------------ training ----
def cg_iterates(normal, b, lam: float, nit: int, keep_at):
    """Plain CG on (normal + lam) x = b from x0 = 0 (torch, FP64 scalars); returns x_nit and the
    residual / iterate pairs {k: (r_k, x_k)} for k in keep_at."""
    import torch
    x = torch.zeros_like(b)
    r = b.clone()
    p = r.clone()
    rr = torch.vdot(r.reshape(-1), r.reshape(-1)).real.double()
    kept = {}
    for k in range(nit + 1):
        if k in keep_at:
            kept[k] = (r.clone(), x.clone())
        if k == nit:
            break
        q = normal(p) + lam * p
        a = rr / torch.vdot(p.reshape(-1), q.reshape(-1)).real.double()
        x = x + a.to(torch.float32) * p
        r = r - a.to(torch.float32) * q
        rn = torch.vdot(r.reshape(-1), r.reshape(-1)).real.double()
        p = r + (rn / rr).to(torch.float32) * p
        rr = rn
    return x, kept


def train(net: PrecondNet, R, E, steps: int = 3000, batch: int = 64, crop: int = 64, margin: int = 6,
          lr: float = 1e-3, lr_min: float = 1e-5, seed: int = 0, log_every: int = 0,
          loss_flags: int = _lib.CNN_LOSS_COS):
    """Adam on random crops of the pairs R[i] -> E[i] (torch complex64 [n, nx, ny] on the device,
    row i the i-th image in (x, y) order); cosine learning-rate decay.  The default loss is the
    scale-invariant one: flexible CG's line search sets the scale of every direction, so only the
    direction of net(r) relative to the error matters.  Returns the loss history."""
    import torch
    g = torch.Generator(device=R.device)
    g.manual_seed(seed)
    n, nx, ny = R.shape
    losses = []
    # crops may reach `margin` pixels past the image (zero there, as the network's own zero
    # padding sees it), so the pixels at the image border are inside some crop's loss mask
    ar = torch.arange(crop, device=R.device)
    for s in range(steps):
        i = torch.randint(0, n, (batch,), generator=g, device=R.device)
        ox = torch.randint(-margin, nx - crop + margin + 1, (batch,), generator=g, device=R.device)
        oy = torch.randint(-margin, ny - crop + margin + 1, (batch,), generator=g, device=R.device)
        ix = (ox[:, None] + ar[None, :])[:, :, None].expand(batch, crop, crop)
        iy = (oy[:, None] + ar[None, :])[:, None, :].expand(batch, crop, crop)
        inside = (ix >= 0) & (ix < nx) & (iy >= 0) & (iy < ny)
        ii = i[:, None, None].expand(batch, crop, crop)
        cx, cy = ix.clamp(0, nx - 1), iy.clamp(0, ny - 1)
        rc = torch.where(inside, R[ii, cx, cy], 0)       # [batch, crop(x), crop(y)]
        ec = torch.where(inside, E[ii, cx, cy], 0)
        # column-major [x, y, batch] views of contiguous [batch, y, x] storage
        rb = rc.permute(0, 2, 1).contiguous().permute(2, 1, 0)
        eb = ec.permute(0, 2, 1).contiguous().permute(2, 1, 0)
        L, _ = net.loss_grad(rb, eb, margin, loss_flags, want_grad=False)
        cur = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * s / max(1, steps - 1)))
        net.adam_step(cur, torch.cuda.current_stream(R.device).cuda_stream)
        losses.append(L)
        if log_every and s % log_every == 0:
            print(f"step {s} loss {L:.4f} lr {cur:.2e}", flush=True)
    return np.array(losses)
