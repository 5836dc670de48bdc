"""findDelAuto: estimate the delay between a measured field trajectory and the MRI data.

Mirrors findDel/findDelAuto.m:1-150 and findDel/interpTrajTime.m:1-28.  The
delay search is a caller of the reconstruction path: every candidate delay
rebuilds the high-order encoding (sampHighOrder, approach 0), reconstructs
the image with cgne through mrSampFunc, and the Gauss-Newton delay update
uses the phase-derivative encoding ``S.setPhiDiv`` (sampHighOrder.m:590-622):

    bhat    = data - A(x)                     (residual)
    bhathat = A_phiDiv(x)                     (d residual / d delay)
    delta  += delJumpFact * real(bhathat \\ bhat)

The coarse search solves its 2*numCoarseSearch+1 candidate delays with the
same iteration count and no stopping rule (findDelAuto.m:76-97); they are
independent, so they run together through ``cgne_batch`` (one CUDA graph
launch per iteration for all candidates).  Trajectory resampling uses the
modified Akima interpolant (MATLAB ``interp1(..., 'makima', NaN)``), which is
restated in ``makima``: Akima's local slopes (H. Akima, J. ACM 17(4), 1970)
with the modified weights w = |d_{i+1} - d_i| + |d_{i+1} + d_i| / 2 that
MATLAB's 'makima' method documents, slopes set to 0 where both weights
vanish, and the two end slopes extrapolated linearly.
"""
from __future__ import annotations

import numpy as np

DERIV_KERNEL = np.array([1 / 8, 1 / 4, 0.0, -1 / 4, -1 / 8])     # findDelAuto.m:70


def _makima_slopes(h, d):
    """Derivatives at the nodes from interval slopes d [n-1, k] (columns independent)."""
    n = d.shape[0] + 1
    if n == 2:
        return np.vstack([d[0], d[0]])
    if n == 3:
        dm1 = 2 * d[0] - d[1]
        dn = 2 * d[-1] - d[-2]
        ext = np.vstack([2 * dm1 - d[0], dm1, d, dn, 2 * dn - d[-1]])
    else:
        d0 = 2 * d[0] - d[1]
        dm1 = 2 * d0 - d[0]
        dn = 2 * d[-1] - d[-2]
        dn1 = 2 * dn - d[-1]
        ext = np.vstack([dm1, d0, d, dn, dn1])
    w = np.abs(np.diff(ext, axis=0)) + np.abs(ext[:-1] + ext[1:]) / 2
    w1 = w[:n]            # |d(i-1) - d(i-2)| + |d(i-1) + d(i-2)| / 2
    w2 = w[2:]            # |d(i+1) - d(i)|   + |d(i+1) + d(i)| / 2
    dl = ext[1:n + 1]     # d(i-1)
    dr = ext[2:n + 2]     # d(i)
    ws = w1 + w2
    with np.errstate(invalid="ignore", divide="ignore"):
        s = (w2 * dl + w1 * dr) / ws
    return np.where(ws == 0, 0.0, s)


def makima(x, y, xq):
    """interp1(x, y, xq, 'makima', NaN) for increasing x; y [n, ...] interpolated along axis 0."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    xq = np.asarray(xq, dtype=np.float64)
    shp = y.shape[1:]
    y2 = y.reshape(y.shape[0], -1)
    h = np.diff(x)
    d = np.diff(y2, axis=0) / h[:, None]
    s = _makima_slopes(h, d)
    i = np.clip(np.searchsorted(x, xq, side="right") - 1, 0, x.size - 2)
    t = (xq - x[i])[:, None]
    hi = h[i][:, None]
    c2 = (3 * d[i] - 2 * s[i] - s[i + 1]) / hi
    c3 = (s[i] + s[i + 1] - 2 * d[i]) / hi ** 2
    out = y2[i] + t * (s[i] + t * (c2 + t * c3))
    out[(xq < x[0]) | (xq > x[-1])] = np.nan
    return out.reshape((xq.size,) + shp)


def interpTrajTime(phs_spha, phs_conc, tdwell_in, delTime, datatime):
    """findDel/interpTrajTime.m: resample [lenTraj x n] trajectories at datatime, delayed by delTime."""
    if phs_spha is None or np.size(phs_spha) == 0:
        if phs_conc is None or np.size(phs_conc) == 0:
            raise ValueError("at least one of phs_spha or phs_conc must be non-empty!")
        lenTraj = np.shape(phs_conc)[0]
    else:
        lenTraj = np.shape(phs_spha)[0]
    trajTim = -delTime + tdwell_in * np.arange(lenTraj)
    dt = np.asarray(datatime, dtype=np.float64).reshape(-1)
    a = None if phs_spha is None or np.size(phs_spha) == 0 else makima(trajTim, phs_spha, dt)
    b = None if phs_conc is None or np.size(phs_conc) == 0 else makima(trajTim, phs_conc, dt)
    return a, b


def _conv_same(a, kern):
    """conv2(a, kern(:), 'same') along axis 0 (odd kernel, zero padding)."""
    K = kern.size
    h = K // 2
    pad = np.zeros((a.shape[0] + 2 * h,) + a.shape[1:])
    pad[h:h + a.shape[0]] = a
    out = np.zeros_like(a, dtype=np.float64)
    for k in range(K):
        out += kern[k] * pad[2 * h - k:2 * h - k + a.shape[0]]
    return out


def _lstsq_scalar(a, b):
    """a(:) \\ b(:) for column vectors: the least-squares scalar."""
    return complex(np.vdot(a, b) / np.vdot(a, a))


def findDelAuto(delSk0, data_in, tdwell, phs_spha, phs_conc, datatime, phs_sph_grid, b0map, Crcvr,
                maxNit_cgne, delJumpFact=3, numCoarseSearch=2, verbose=False):
    """[delSk, delSk_perIt] = findDelAuto(delSk0, data_in, tdwell, phs_spha, phs_conc, datatime,
    phs_sph_grid, b0map, Crcvr, maxNit_cgne, delJumpFact, numCoarseSearch)  (findDelAuto.m:1-150).

    phs_spha [lenTraj x nspha], phs_conc [lenTraj x nconc] sampled every tdwell from t = 0;
    datatime [M]; data_in [M x C] (numpy or a CUDA tensor); Crcvr [imN, (1,) C].
    Returns the delay and the per-iteration history (first entry: after the coarse search).
    """
    from .ops import rcvrOp, sampHighOrder
    from .sense import mrSampOp
    from .solvers import cgne, cgne_batch

    def log(s):
        if verbose:
            print(s, end="", flush=True)

    b0map = np.asarray(b0map, dtype=np.float64)
    imN = list(b0map.shape)
    maps = np.asarray(Crcvr).reshape(imN + [-1], order="F")
    R = rcvrOp(maps, 0)
    datatime = np.asarray(datatime, dtype=np.float64).reshape(-1)
    dtsamp = datatime[1] - datatime[0]
    phs_spha = np.asarray(phs_spha, dtype=np.float64)
    phs_conc = np.zeros((phs_spha.shape[0], 0)) if phs_conc is None else np.asarray(phs_conc, dtype=np.float64)
    dspha_dt = _conv_same(phs_spha, DERIV_KERNEL) / tdwell                      # findDelAuto.m:71-72
    dconc_dt = _conv_same(phs_conc, DERIV_KERNEL) / tdwell
    data = data_in
    host = not (type(data).__module__.startswith("torch"))
    dvec = np.asarray(data).reshape(-1, order="F") if host else None

    def operator(delSk):
        sp, cc = interpTrajTime(phs_spha, phs_conc, tdwell, delSk, datatime)        # 81, 111
        cc = np.zeros((0, datatime.size)) if cc is None else cc.T
        S = sampHighOrder(b0map, datatime, sp.T, cc, phs_sph_grid, None, 1, 0, 0)   # 84, 115 (approach 0)
        return S, mrSampOp(S, R)

    log(f"findDelAuto: Init guess {delSk0:.2f}; ")
    if numCoarseSearch > 0:                                                     # 76-97
        log(f"coarse search (N={2 * numCoarseSearch + 1})")
        cands = [delSk0 + c * dtsamp for c in range(-numCoarseSearch, numCoarseSearch + 1)]
        ops = [operator(d)[1] for d in cands]
        _, infos = cgne_batch(ops, [data] * len(ops), maxNit_cgne, {"stopOnResInc": 0})
        last = [info["resSqAll"][-1] for info in infos]
        delSk = cands[int(np.argmin(last))]          # first minimum, as the strict '<' update keeps it
        log(f" {delSk:.2f}; ")
    else:
        delSk = delSk0
    ntry = 0
    delChange = np.inf
    delThresh = 0.005                                                           # 104
    delChangePrev = 0.0
    perIt = [delSk]
    log("iterations...")
    nit = maxNit_cgne
    resvec = None
    while abs(delChange) > delThresh:                                           # 108-148
        _, dd_c = interpTrajTime(None, dconc_dt, tdwell, delSk, datatime) if dconc_dt.size else (None, None)
        dd_s, _ = interpTrajTime(dspha_dt, None, tdwell, delSk, datatime)
        S, A = operator(delSk)
        if ntry > 0:
            nit = len(resvec) - 1                                               # 116-120
        x, resvec, *_ = cgne(A, data, None, nit, {"stopOnResInc": 1 if ntry == 0 else 0})   # 121
        Ax = A(x, "notransp")
        Sd = S.setPhiDiv(dd_s.T, np.zeros((0, datatime.size)) if dd_c is None else dd_c.T)
        bhathat = mrSampOp(Sd, R)(x, "notransp")                                # 124-128
        if host:
            bhat = dvec - np.asarray(Ax).reshape(-1, order="F")
            bh = np.asarray(bhathat).reshape(-1, order="F")
        else:
            bhat = (data - Ax).reshape(-1).cpu().numpy()
            bh = bhathat.reshape(-1).cpu().numpy()
        delChange = delJumpFact * _lstsq_scalar(bh, bhat).real                  # 130-131
        delSk = delSk + delChange
        log(f" {delSk:.2f},")
        if ntry > 0 and np.sign(delChangePrev) != np.sign(delChange) and delJumpFact > 1:   # 134-136
            delJumpFact = delJumpFact / 2
        delChangePrev = delChange
        ntry += 1
        perIt.append(delSk)
        if ntry > 50:
            import warnings
            warnings.warn(f"did not converge after {ntry} iterations")
            break
    log(" done\n")
    return delSk, np.asarray(perIt)
