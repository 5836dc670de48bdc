"""FP64 restatement of ``@sampHighOrder`` direct/segmented encoding (TEST ORACLE).

* ``basis_harm``   — computeHarmonics/basisFuncHarm.m:24-96 (terms 1..36)
* ``basis_conc``   — computeHarmonics/basisFuncConc.m:13-23 (terms 1..4)
* ``ShoRef``       — operators/@sampHighOrder/sampHighOrder.m: constructor
  (129-291), ``prepForDirect`` (496-588), ``useDirectWorker`` (361-391),
  ``useSegmentedWorker`` (393-457), with the phase-derivative variant of
  ``setPhiDiv`` (590-622, used at 375-382).

The phase matrix ``kbase[v, m]`` (voxels x samples, column-major voxel order)
is built in FP64; forward is ``exp(+i kbase.') x / sqrt(V)``, adjoint is
``exp(-i kbase) y / sqrt(V)``.  Large problems are evaluated in sample
chunks so that the oracle never materialises V x M at once.
Test infrastructure only; see ``oracle/__init__.py``.
"""
from __future__ import annotations

import math

import numpy as np


def basis_harm(x, y, z, n):
    """basisFuncHarm.m:24-96 for one index n (1-based)."""
    r2 = x ** 2 + y ** 2 + z ** 2
    f = {
        1: lambda: np.ones_like(x),
        2: lambda: x,
        3: lambda: y,
        4: lambda: z,
        5: lambda: x * y,
        6: lambda: z * y,
        7: lambda: 3 * z ** 2 - r2,
        8: lambda: x * z,
        9: lambda: x ** 2 - y ** 2,
        10: lambda: 3 * y * x ** 2 - y ** 3,
        11: lambda: x * z * y,
        12: lambda: (5 * z ** 2 - r2) * y,
        13: lambda: 5 * z ** 3 - 3 * z * r2,
        14: lambda: (5 * z ** 2 - r2) * x,
        15: lambda: x ** 2 * z - y ** 2 * z,
        16: lambda: x ** 3 - 3 * x * y ** 2,
        17: lambda: (x * y) * (x ** 2 - y ** 2),
        18: lambda: (y * z) * (3 * x ** 2 - y ** 2),
        19: lambda: (x * y) * (7 * z ** 2 - r2),
        20: lambda: y * (7 * z ** 3 - 3 * z * r2),
        21: lambda: 35 * z ** 4 - 30 * z ** 2 * r2 + 3 * r2 ** 2,
        22: lambda: x * (7 * z ** 3 - 3 * z * r2),
        23: lambda: (x ** 2 - y ** 2) * (7 * z ** 2 - r2),
        24: lambda: x * (x ** 2 - 3 * y ** 2) * z,
        25: lambda: x ** 2 * (x ** 2 - 3 * y ** 2) - y ** 2 * (3 * x ** 2 - y ** 2),
        26: lambda: y * (5 * x ** 4 - 10 * x ** 2 * y ** 2 + y ** 4),
        27: lambda: x * y * z * (x ** 2 - y ** 2),
        28: lambda: y * (r2 - 9 * z ** 2) * (y ** 2 - 3 * x ** 2),
        29: lambda: x * y * z * (3 * z ** 2 - r2),
        30: lambda: y * (r2 ** 2 - 14 * r2 * z ** 2 + 21 * z ** 4),
        31: lambda: 63 * z ** 5 - 70 * z ** 3 * r2 + 15 * z * r2 ** 2,
        32: lambda: x * (r2 ** 2 - 14 * r2 * z ** 2 + 21 * z ** 4),
        33: lambda: z * (3 * z ** 2 - r2) * (x ** 2 - y ** 2),
        34: lambda: x * (r2 - 9 * z ** 2) * (3 * y ** 2 - x ** 2),
        35: lambda: z * (x ** 4 - 6 * x ** 2 * y ** 2 + y ** 4),
        36: lambda: x ** 5 - 10 * x ** 3 * y ** 2 + 5 * x * y ** 4,
    }
    if n not in f:
        raise ValueError("Basis function undefined.")
    return f[n]()


def basis_conc(x, y, z, n):
    """basisFuncConc.m:13-23."""
    if n == 1:
        return z * z
    if n == 2:
        return x * x + y * y
    if n == 3:
        return x * z
    if n == 4:
        return y * z
    raise ValueError("Basis function undefined.")


class ShoRef:
    """FP64 sampHighOrder with approach 0 (direct); segmented gives the same sums."""

    def __init__(self, b0, sampTimes, phs_spha, phs_conc, grid, b0mask=None):
        gx = np.asarray(grid["x"], dtype=np.float64)
        self.imSize = gx.shape if not (gx.ndim == 2 and gx.shape[1] == 1) else (gx.shape[0],)
        self.V = gx.size
        self.x = gx.reshape(-1, order="F")
        self.y = np.asarray(grid["y"], dtype=np.float64).reshape(-1, order="F")
        self.z = np.asarray(grid["z"], dtype=np.float64).reshape(-1, order="F")
        self.b0 = np.zeros(self.V) if b0 is None or np.size(b0) == 0 else \
            np.asarray(b0, dtype=np.float64).reshape(-1, order="F")          # 221-227
        self.t = np.asarray(sampTimes, dtype=np.float64)
        self.kSize = self.t.shape if not (self.t.ndim == 2 and self.t.shape[1] == 1) else (self.t.shape[0],)
        self.t = self.t.reshape(-1, order="F")
        self.M = self.t.size
        ps = np.asarray(phs_spha, dtype=np.float64)
        self.phs_spha = ps.reshape(ps.shape[0], -1, order="F")
        pc = np.asarray(phs_conc, dtype=np.float64) if phs_conc is not None and np.size(phs_conc) else np.zeros((0, self.M))
        self.phs_conc = pc.reshape(pc.shape[0], self.M, order="F")
        self.b0mask = None if b0mask is None or np.size(b0mask) == 0 else \
            np.asarray(b0mask, dtype=np.float64).reshape(-1, order="F")
        self.adjoint = False
        self.ksphaDiv = None
        self.kconcDiv = None

    def ctranspose(self):
        o = ShoRef.__new__(ShoRef)
        o.__dict__.update(self.__dict__)
        o.adjoint = not self.adjoint
        return o

    @property
    def H(self):
        return self.ctranspose()

    def basis_matrix(self, spha=None, conc=None, with_b0=True):
        """Spatial basis B [V, K] and temporal coefficients P [K, M] with kbase = B @ P.

        Follows prepForDirect (sampHighOrder.m:558-586): terms n > 4 and the
        concomitant terms are multiplied by ``b0mask`` when given; the B0
        term is ``b0 .* b0mask`` times the sample times.
        """
        spha = self.phs_spha if spha is None else spha
        conc = self.phs_conc if conc is None else conc
        cols, rows = [], []
        for n in range(1, spha.shape[0] + 1):                            # 560-569
            bf = basis_harm(self.x, self.y, self.z, n)
            if n > 4 and self.b0mask is not None:
                bf = bf * self.b0mask
            cols.append(bf)
            rows.append(spha[n - 1])
        for n in range(1, conc.shape[0] + 1):                            # 570-579
            bf = basis_conc(self.x, self.y, self.z, n)
            if self.b0mask is not None:
                bf = bf * self.b0mask
            cols.append(bf)
            rows.append(conc[n - 1])
        if with_b0 and self.M > 1:                                       # 580-586
            b0a = self.b0 * self.b0mask if self.b0mask is not None else self.b0
            cols.append(b0a)
            rows.append(self.t)
        return np.stack(cols, axis=1), np.stack(rows, axis=0)

    def kbase(self, m0=0, m1=None):
        B, P = self.basis_matrix()
        return B @ P[:, m0:m1]

    def setPhiDiv(self, ksphaDiv, kconcDiv):
        """sampHighOrder.m:590-622 (phase-derivative forward operator)."""
        o = self.ctranspose().ctranspose()
        o.ksphaDiv = np.asarray(ksphaDiv, dtype=np.float64).reshape(np.shape(ksphaDiv)[0], self.M, order="F")
        o.kconcDiv = np.asarray(kconcDiv, dtype=np.float64).reshape(np.shape(kconcDiv)[0], self.M, order="F")
        return o

    def mtimes(self, x, chunk=1024):
        """useDirectWorker (sampHighOrder.m:361-391); evaluated in sample chunks."""
        x = np.asarray(x)
        B, P = self.basis_matrix()
        if self.ksphaDiv is not None:
            Bd, Pd = self.basis_matrix(self.ksphaDiv, self.kconcDiv, with_b0=False)
        s = 1.0 / math.sqrt(self.V)                                      # 387
        if self.adjoint:
            nk = len(self.kSize)
            extra = x.shape[nk:]
            yv = x.reshape(self.M, -1, order="F").astype(np.complex128)
            out = np.zeros((self.V, yv.shape[1]), dtype=np.complex128)
            for m0 in range(0, self.M, chunk):
                ph = B @ P[:, m0:m0 + chunk]
                out += np.exp(-1j * ph) @ yv[m0:m0 + chunk]              # 371
            return (out * s).reshape(list(self.imSize) + list(extra), order="F")
        ni = len(self.imSize)
        extra = x.shape[ni:]
        xv = x.reshape(self.V, -1, order="F").astype(np.complex128)
        out = np.empty((self.M, xv.shape[1]), dtype=np.complex128)
        for m0 in range(0, self.M, chunk):
            ph = B @ P[:, m0:m0 + chunk]
            E = np.exp(1j * ph)
            if self.ksphaDiv is not None:                                # 378-380
                E = 1j * E * (Bd @ Pd[:, m0:m0 + chunk])
            out[m0:m0 + chunk] = E.T @ xv                                 # 376
        return (out * s).reshape(list(self.kSize) + list(extra), order="F")

    __mul__ = lambda self, x: self.mtimes(x)
