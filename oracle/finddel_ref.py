"""FP64 restatement of findDel/findDelAuto.m:1-150 and findDel/interpTrajTime.m:1-28 (TEST ORACLE).

The encoding of each candidate delay is the direct ``ShoRef`` (approach 0,
findDelAuto.m:66), the image update is ``cgne_ref`` through ``mrsampfunc``
(findDelAuto.m:83-88, 113-121), and the delay update uses the
phase-derivative encoding ``ShoRef.setPhiDiv`` (124-131).  Trajectory
resampling is ``interp1(..., 'makima', NaN)``, evaluated here with SciPy's
modified Akima interpolant (``Akima1DInterpolator(method='makima')``, which
implements the same published rule as MATLAB's 'makima').
Test infrastructure only; see ``oracle/__init__.py``.
"""
from __future__ import annotations

import numpy as np

from .sense_ref import RcvrRef, cgne_ref, mrsampfunc
from .sho_ref import ShoRef


def interp_traj_time(phs_spha, phs_conc, tdwell_in, delTime, datatime):
    """interpTrajTime.m:12-27."""
    from scipy.interpolate import Akima1DInterpolator
    lenTraj = np.shape(phs_spha)[0] if phs_spha is not None and np.size(phs_spha) else np.shape(phs_conc)[0]
    trajTim = -delTime + tdwell_in * np.arange(lenTraj)                  # 21
    dt = np.asarray(datatime, dtype=np.float64).reshape(-1)
    f = lambda a: Akima1DInterpolator(trajTim, a, method="makima", extrapolate=False)(dt)
    a = f(phs_spha) if phs_spha is not None and np.size(phs_spha) else None    # 22-24
    b = f(phs_conc) if phs_conc is not None and np.size(phs_conc) else None    # 25-27
    return a, b


def deriv_same(a, tdwell):
    """conv2(a, [1/8 1/4 0 -1/4 -1/8]', 'same') / tdwell along time (findDelAuto.m:70-72)."""
    kern = np.array([1 / 8, 1 / 4, 0.0, -1 / 4, -1 / 8])
    full = np.zeros((a.shape[0] + kern.size - 1,) + a.shape[1:])
    for k in range(kern.size):                   # full convolution, then the central part
        full[k:k + a.shape[0]] += kern[k] * a
    h = kern.size // 2
    return full[h:h + a.shape[0]] / tdwell


def find_del_auto(delSk0, data_in, tdwell, phs_spha, phs_conc, datatime, grid, b0map, Crcvr, maxNit_cgne,
                  delJumpFact=3, numCoarseSearch=2):
    """findDelAuto.m:1-150; returns (delSk, delSk_perIt)."""
    b0map = np.asarray(b0map, dtype=np.float64)
    imN = list(b0map.shape)
    R = RcvrRef(np.asarray(Crcvr).reshape(imN + [-1], order="F"))     # 61-65
    datatime = np.asarray(datatime, dtype=np.float64).reshape(-1)
    dtsamp = datatime[1] - datatime[0]                                     # 67
    dspha = deriv_same(phs_spha, tdwell)                                   # 71
    dconc = deriv_same(phs_conc, tdwell)                                   # 72
    M = datatime.size

    def op(delSk):
        sp, cc = interp_traj_time(phs_spha, phs_conc, tdwell, delSk, datatime)
        cc = np.zeros((0, M)) if cc is None else cc.T
        S = ShoRef(b0map, datatime, sp.T, cc, grid)
        return S, (lambda x, t: mrsampfunc(x, t, S, R))

    if numCoarseSearch > 0:                                                # 76-97
        resmin = np.inf
        for c in range(-numCoarseSearch, numCoarseSearch + 1):
            d = delSk0 + c * dtsamp
            _, f = op(d)
            _, resvec, *_ = cgne_ref(f, data_in, None, maxNit_cgne, {"stopOnResInc": 0})
            if resvec[-1] < resmin:
                delmin, resmin = d, resvec[-1]
        delSk = delmin
    else:
        delSk = delSk0
    ntry, delChange, delThresh, prev = 0, np.inf, 0.005, 0.0               # 101-104
    perIt = [delSk]
    nit = maxNit_cgne
    resvec = None
    while abs(delChange) > delThresh:                                      # 108
        dd_s, dd_c = interp_traj_time(dspha, dconc if np.size(dconc) else None, tdwell, delSk, datatime)
        S, f = op(delSk)
        if ntry > 0:
            nit = len(resvec) - 1                                          # 116-120
        x, resvec, *_ = cgne_ref(f, data_in, None, nit, {"stopOnResInc": 1 if ntry == 0 else 0})
        bhat = data_in - f(x, "notransp")                                  # 124
        Sd = S.setPhiDiv(dd_s.T, np.zeros((0, M)) if dd_c is None else dd_c.T)
        bhathat = mrsampfunc(x, "notransp", Sd, R)                          # 126-128
        a, b = bhathat.reshape(-1, order="F"), bhat.reshape(-1, order="F")
        delChange = delJumpFact * (np.vdot(a, b) / np.vdot(a, a)).real     # 130-131
        delSk = delSk + delChange
        if ntry > 0 and np.sign(prev) != np.sign(delChange) and delJumpFact > 1:   # 134-136
            delJumpFact = delJumpFact / 2
        prev = delChange
        ntry += 1
        perIt.append(delSk)
        if ntry > 50:                                                       # 140-143
            break
    return delSk, np.asarray(perIt)
