"""matmri_gb300 — GB300-native (sm_103a) MatMRI reconstruction hot path.

Drop-in classes and functions with the reference's names and arguments:
``nufftOp``, ``rcvrOp``, ``sampHighOrder``, ``mrSampFunc`` (+ ``mrSampOp``),
``cgne``, ``powermethod``, ``bfista``, ``dwtND``, ``findDelAuto``,
``interpTrajTime``, ``mrSampFuncMat`` (+ ``dense_solve``).  All compute runs in
``libmatmri_gb300.so`` (hand-written CUDA for sm_103a behind a C ABI); the
package raises on import of an operator when the library is missing.
"""
from ._lib import MatmriError, check_device_error, load as load_library
from .ops import nufftOp, rcvrOp, sampHighOrder
from .sense import mrSampFunc, mrSampOp
from .solvers import bfista, cgne, cgne_batch, dwtND, powermethod
from .learned import PrecondNet, lpcg
from .finddel import findDelAuto, interpTrajTime
from .densemat import dense_solve, mrSampFuncMat

__all__ = ["nufftOp", "rcvrOp", "sampHighOrder", "mrSampFunc", "mrSampOp", "cgne", "cgne_batch", "powermethod",
           "bfista", "dwtND", "PrecondNet", "lpcg", "findDelAuto", "interpTrajTime", "mrSampFuncMat",
           "dense_solve", "MatmriError", "check_device_error", "load_library"]
