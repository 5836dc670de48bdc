"""FP64 restatement of operators/mrSampFuncMat.m:22-47 (TEST ORACLE).

``AtA = sum_c conj(r_c) r_c.' .* (S' * S)`` with
``S = exp(1i*kbase(mask, :)).' / sqrt(nnz(mask))`` and ``Aty = R'*(S'*y)``
on the mask.  The reference casts kbase to single before the exponential
(mrSampFuncMat.m:35); the oracle keeps FP64 throughout.
Test infrastructure only; see ``oracle/__init__.py``.
"""
from __future__ import annotations

import numpy as np

from .sense_ref import RcvrRef
from .sho_ref import ShoRef


def mrsampfuncmat_ref(y, Crcvr, b0, sampTimes, phs_spha, phs_conc, grid, imMask=None):
    S = ShoRef(b0, sampTimes, phs_spha, phs_conc, grid)                  # 24
    b0a = np.asarray(b0)
    maps = np.asarray(Crcvr).reshape(list(b0a.shape) + [-1], order="F")
    R = RcvrRef(maps)                                                     # 27
    mask = np.ones(b0a.shape, bool) if imMask is None else np.asarray(imMask) > 0
    m = mask.reshape(-1, order="F")
    Aty = R.H.mtimes(S.H.mtimes(y)).reshape(-1, order="F")[m]             # 30-31
    k = S.kbase()[m]                                                      # [Vm, M]
    Sm = np.exp(1j * k).T / np.sqrt(Aty.size)                             # 35-37
    G = Sm.conj().T @ Sm                                                  # 38
    r = maps.reshape(-1, maps.shape[-1], order="F")[m]                    # [Vm, C]
    AtA = np.zeros_like(G)
    for c in range(r.shape[1]):                                           # 40-45
        AtA += np.conj(r[:, c])[:, None] * G * r[:, c][None, :]
    return AtA, Aty
