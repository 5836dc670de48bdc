"""Array plumbing between Python callers and the C ABI.

Arrays keep MATLAB index semantics (``x[i1, i2, ..., extra]``) and are handed
to the library as column-major interleaved complex64 — the layout MATLAB's
interleaved-complex API gives a MEX file.  numpy arrays are passed as host
pointers (the library stages them through device memory); CUDA torch tensors
are passed as device pointers without a copy when they already are
column-major complex64.
"""
from __future__ import annotations

import numpy as np


def _torch():
    import torch  # noqa: WPS433 (optional dependency)
    return torch


def is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


class Buf:
    """A column-major complex64 view of an input, kept alive for the call."""

    __slots__ = ("obj", "ptr", "shape", "kind", "device", "double")

    def __init__(self, obj, ptr, shape, kind, device=None, double=False):
        self.obj, self.ptr, self.shape, self.kind, self.device, self.double = obj, ptr, shape, kind, device, double


def as_c64(x) -> Buf:
    if is_torch(x):
        torch = _torch()
        double = x.dtype in (torch.float64, torch.complex128)
        t = x.to(torch.complex64)
        rev = tuple(range(t.dim() - 1, -1, -1))
        if t.dim() > 1:
            t = t.permute(rev).contiguous().permute(rev)
        else:
            t = t.contiguous()
        return Buf(t, t.data_ptr(), tuple(t.shape), "torch", t.device, double)
    a = np.asarray(x)
    double = a.dtype in (np.float64, np.complex128) or a.dtype.kind in "iub"
    a = np.asfortranarray(a, dtype=np.complex64)
    return Buf(a, a.ctypes.data, a.shape, "np", None, double)


def alloc_like(b: Buf, shape):
    shape = tuple(int(s) for s in shape)
    if b.kind == "torch":
        torch = _torch()
        t = torch.empty(shape[::-1], dtype=torch.complex64, device=b.device)
        if len(shape) > 1:
            t = t.permute(tuple(range(len(shape) - 1, -1, -1)))
        return t, t.data_ptr()
    a = np.empty(shape, dtype=np.complex64, order="F")
    return a, a.ctypes.data


def finish(out, b: Buf):
    """Reverts to double precision when the input was double (nufftOp.m:404-406)."""
    if not b.double:
        return out
    if b.kind == "torch":
        return out.to(_torch().complex128)
    return out.astype(np.complex128)


def stream_of(b: Buf):
    """Current torch stream for device inputs (NULL = legacy default stream)."""
    if b.kind == "torch" and b.device is not None and b.device.type == "cuda":
        return _torch().cuda.current_stream(b.device).cuda_stream
    return None


def f64(x, n=None):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1, order="F"))
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a
