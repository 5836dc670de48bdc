"""Dense normal matrix of the high-order encoding and its direct solve.

``mrSampFuncMat`` mirrors operators/mrSampFuncMat.m:1-47: it returns
``AtA = R'*S'*S*R`` restricted to ``imMask`` as a dense device matrix (built
by ``mmr_dense_normal``: encoding matrix from the phase table, a cuBLAS Gram
GEMM, the coil weighting as an in-place epilogue) and ``Aty = R'*(S'*y)`` on
the mask.  Note the reference's scaling: the Gram is normalised by the number
of mask voxels (mrSampFuncMat.m:37) while ``Aty`` carries sampHighOrder's
``1/sqrt(numel(b0))`` (sampHighOrder.m:387); the two agree for a full mask.
``dense_solve`` is the demo's ``(AtA + lam2*I) \\ Aty`` (demos/demo_denseMat.m:98-106).
The matrix is returned as a CUDA torch tensor with MATLAB index semantics
(``AtA[v, w]``), stored column-major.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _torch():
    import torch
    return torch


def mrSampFuncMat(y, Crcvr, b0, sampTimes, phs_spha, phs_conc, phs_grid, imMask=None):
    """[AtA, Aty] = mrSampFuncMat(y, Crcvr, b0, sampTimes, phs_spha, phs_conc, phs_grid, imMask)."""
    torch = _torch()
    from .ops import rcvrOp, sampHighOrder
    from .sense import mrSampOp
    S = sampHighOrder(b0, sampTimes, phs_spha, phs_conc, phs_grid)               # mrSampFuncMat.m:24
    b0a = np.asarray(b0)
    maps = np.asarray(Crcvr).reshape(list(b0a.shape) + [-1], order="F")
    R = rcvrOp(maps, 0)                                                           # 27
    mask = np.ones(b0a.shape, dtype=bool) if imMask is None else np.asarray(imMask) > 0
    vox = np.ascontiguousarray(np.flatnonzero(mask.reshape(-1, order="F")).astype(np.int64))
    n = vox.size
    dev = torch.device("cuda", torch.cuda.current_device())
    Aty = mrSampOp(S, R)(y, "transp")                                             # 30
    if type(Aty).__module__.startswith("torch"):                                  # 31: Aty(imMask(:))
        flat = Aty.T.reshape(-1) if Aty.dim() > 1 else Aty
        Aty = flat[torch.from_numpy(vox).to(Aty.device)].to(torch.complex64)
    else:
        Aty = torch.from_numpy(np.ascontiguousarray(np.asarray(Aty).reshape(-1, order="F")[vox],
                                                    dtype=np.complex64)).to(dev)
    At = torch.empty((n, n), dtype=torch.complex64, device=dev)                  # column-major storage
    lib = _lib.load()
    _lib.check(lib.mmr_dense_normal(S.handle, R.handle, vox.ctypes.data_as(C.POINTER(C.c_int64)), n,
                                    At.data_ptr(), torch.cuda.current_stream(dev).cuda_stream))
    return At.T, Aty


def dense_solve(AtA, Aty, lam2=0.0):
    """x = (AtA + lam2*I) \\ Aty on the device; returns (x, method) with method 'chol' or 'lu'."""
    torch = _torch()
    n = AtA.shape[0]
    if AtA.shape != (n, n):
        raise ValueError("AtA must be square")
    cm = AtA.T                     # column-major storage of AtA[v, w]
    if not cm.is_contiguous():
        cm = cm.contiguous()
    b = Aty.reshape(-1).to(torch.complex64).contiguous()
    if b.numel() != n:
        raise ValueError("Aty must have one entry per row of AtA")
    x = torch.empty_like(b)
    m = C.c_int32(0)
    lib = _lib.load()
    _lib.check(lib.mmr_dense_solve(cm.data_ptr(), n, float(lam2), b.data_ptr(), x.data_ptr(), C.byref(m),
                                   torch.cuda.current_stream(b.device).cuda_stream))
    return x, ("chol" if m.value == 1 else "lu")
