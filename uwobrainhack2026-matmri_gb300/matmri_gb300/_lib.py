"""ctypes binding of libmatmri_gb300.so (the C ABI in include/matmri_gb300.h).

The library is required: importing the operators without it raises
immediately — there is no CPU fallback path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmatmri_gb300.so")

MMR_OK = 0
ERR_NAMES = {1: "BADARG", 2: "NOMEM", 3: "CUDA", 4: "TIMEOUT", 5: "NONFINITE", 6: "UNSUPPORTED"}


class MatmriError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"matmri:gb300:{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


class NufftDesc(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("imN", C.c_int64 * 3), ("nsamp", C.c_int64),
                ("kloc", C.POINTER(C.c_double)), ("dcf", C.POINTER(C.c_double)),
                ("os", C.c_double), ("kwidth", C.c_int32)]


class ShoDesc(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("imN", C.c_int64 * 3), ("nsamp", C.c_int64),
                ("nspha", C.c_int32), ("nconc", C.c_int32),
                ("b0", C.POINTER(C.c_double)), ("t", C.POINTER(C.c_double)),
                ("spha", C.POINTER(C.c_double)), ("conc", C.POINTER(C.c_double)),
                ("gx", C.POINTER(C.c_double)), ("gy", C.POINTER(C.c_double)),
                ("gz", C.POINTER(C.c_double)), ("mask", C.POINTER(C.c_double))]


class ShoInterpDesc(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("imN", C.c_int64 * 3), ("nsamp", C.c_int64), ("nterms", C.c_int32),
                ("kloc", C.POINTER(C.c_double)), ("svd_space", C.POINTER(C.c_double)),
                ("svd_time", C.POINTER(C.c_double)), ("phs_shift", C.POINTER(C.c_double)),
                ("os", C.c_double), ("kwidth", C.c_int32)]


class SenseDesc(C.Structure):
    _fields_ = [("nufft", C.c_void_p), ("sho", C.c_void_p), ("rcvr", C.c_void_p),
                ("W", C.POINTER(C.c_float)), ("w_per_coil", C.c_int32), ("tikreg", C.c_double)]


class Tuning(C.Structure):
    _fields_ = [("coil_chunk", C.c_int32), ("tile", C.c_int32), ("coil_group", C.c_int32), ("item", C.c_int32),
                ("fft_lines", C.c_int32), ("normal_mode", C.c_int32)]


class CgneOpts(C.Structure):
    _fields_ = [("nit_max", C.c_int32), ("res_thresh", C.c_double), ("res_change_thresh", C.c_double),
                ("x_change_thresh", C.c_double), ("exp_res_n", C.c_int32), ("nse_thresh_fact", C.c_double),
                ("nse_extra_it", C.c_int32), ("stop_on_res_inc", C.c_int32), ("res_inc_thresh", C.c_double),
                ("stop_on_xdif_inc", C.c_int32), ("noise_var", C.c_double), ("noise", C.c_void_p),
                ("noise_seed", C.c_uint64), ("gtruth", C.c_void_p), ("tik_diag", C.POINTER(C.c_float)),
                ("w_per_coil", C.c_int32), ("want_history", C.c_int32)]


class CgneHist(C.Structure):
    _fields_ = [("res_sq", C.POINTER(C.c_double)), ("mse", C.POINTER(C.c_double)),
                ("xnorm", C.POINTER(C.c_double)), ("xdiff", C.POINTER(C.c_double)),
                ("capacity", C.c_int32), ("n", C.c_int32), ("stop_thresh", C.c_double),
                ("status", C.c_int32), ("nit", C.c_int32)]


class BfistaOpts(C.Structure):
    _fields_ = [("nit_max", C.c_int32), ("res_thresh", C.c_double), ("max_eig", C.c_double),
                ("n_restart", C.c_int32), ("x_mask", C.c_void_p)]


class BfistaHist(C.Structure):
    _fields_ = [("res_sq", C.POINTER(C.c_double)), ("rx", C.POINTER(C.c_double)),
                ("test", C.POINTER(C.c_double)), ("capacity", C.c_int32), ("n", C.c_int32),
                ("max_eig", C.c_double)]


class LpcgOpts(C.Structure):
    _fields_ = [("nit_max", C.c_int32), ("tol", C.c_double), ("tik_diag", C.POINTER(C.c_float)),
                ("lam", C.c_double), ("gtruth", C.c_void_p), ("stall_window", C.c_int32), ("flags", C.c_int32),
                ("poll", C.c_int32), ("fcg_m", C.c_int32)]


class LpcgHist(C.Structure):
    _fields_ = [("res_sq", C.POINTER(C.c_double)), ("err_sq", C.POINTER(C.c_double)), ("capacity", C.c_int32),
                ("n", C.c_int32), ("nit", C.c_int32), ("status", C.c_int32), ("fell_back_at", C.c_int32),
                ("true_res_rel", C.c_double)]


CNN_FP32_ACT = 1
CNN_TENSOR = 2
CNN_LOSS_COS = 4
CNN_LINEAR = 8
CNN_FOLDED = 16

# name -> (restype, argtypes)
SIGNATURES = {
    "mmr_abi_version": (C.c_int, []),
    "mmr_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "mmr_device_info": (C.c_int, [C.POINTER(C.c_int)] * 4),
    "mmr_check_device_error": (C.c_int, [C.c_void_p]),
    "mmr_debug_set_wait_polls": (C.c_int, [C.c_int32]),
    "mmr_kernel_launches": (C.c_int, [C.POINTER(C.c_uint64)]),
    "mmr_sense_profile_normal": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_double),
                                           C.POINTER(C.c_int32), C.c_void_p]),
    "mmr_nufft_create": (C.c_int, [C.POINTER(NufftDesc), C.POINTER(C.c_void_p)]),
    "mmr_nufft_set_dcf": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "mmr_nufft_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "mmr_nufft_apply": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "mmr_nufft_prep_toep": (C.c_int, [C.c_void_p, C.c_double, C.c_int32]),
    "mmr_nufft_destroy": (C.c_int, [C.c_void_p]),
    "mmr_nufft_adjoint_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "mmr_rcvr_create": (C.c_int, [C.c_int32, C.POINTER(C.c_int64), C.c_int64, C.c_void_p, C.POINTER(C.c_void_p)]),
    "mmr_rcvr_apply": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mmr_rcvr_destroy": (C.c_int, [C.c_void_p]),
    "mmr_sho_create": (C.c_int, [C.POINTER(ShoDesc), C.POINTER(C.c_void_p)]),
    "mmr_sho_apply": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "mmr_sho_destroy": (C.c_int, [C.c_void_p]),
    "mmr_sho_set_tensor": (C.c_int, [C.c_void_p, C.c_int]),
    "mmr_sho_kbase": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mmr_sho_interp_create": (C.c_int, [C.POINTER(ShoInterpDesc), C.POINTER(C.c_void_p)]),
    "mmr_dense_normal": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int64), C.c_int64, C.c_void_p,
                                   C.c_void_p]),
    "mmr_dense_solve": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_void_p,
                                  C.POINTER(C.c_int32), C.c_void_p]),
    "mmr_sho_phidiv_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.POINTER(C.c_void_p)]),
    "mmr_sense_create": (C.c_int, [C.POINTER(SenseDesc), C.POINTER(C.c_void_p)]),
    "mmr_sense_apply": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mmr_sense_normal": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mmr_sense_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "mmr_sense_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "mmr_sense_destroy": (C.c_int, [C.c_void_p]),
    "mmr_cgne_default_opts": (C.c_int, [C.POINTER(CgneOpts)]),
    "mmr_cgne_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_float), C.POINTER(CgneOpts),
                                 C.c_void_p, C.POINTER(CgneHist), C.c_void_p]),
    "mmr_cgne_solve_batch": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p),
                                       C.POINTER(C.c_void_p), C.POINTER(CgneOpts), C.POINTER(CgneHist), C.c_void_p]),
    "mmr_powermethod": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), C.c_void_p]),
    "mmr_dwt_haar": (C.c_int, [C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int, C.c_void_p,
                               C.c_void_p, C.c_void_p]),
    "mmr_bfista_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_float), C.c_int32,
                                   C.c_void_p, C.POINTER(BfistaOpts), C.c_void_p, C.POINTER(BfistaHist),
                                   C.c_void_p]),
    "mmr_cnn_create": (C.c_int, [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_void_p)]),
    "mmr_cnn_num_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "mmr_cnn_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mmr_cnn_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mmr_cnn_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int32,
                                  C.c_void_p]),
    "mmr_cnn_loss_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int32,
                                    C.c_int32, C.POINTER(C.c_double), C.c_void_p, C.c_void_p]),
    "mmr_cnn_adam_step": (C.c_int, [C.c_void_p, C.c_float, C.c_void_p]),
    "mmr_cnn_destroy": (C.c_int, [C.c_void_p]),
    "mmr_lpcg_default_opts": (C.c_int, [C.POINTER(LpcgOpts)]),
    "mmr_lpcg_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(LpcgOpts), C.c_void_p,
                                 C.POINTER(LpcgHist), C.c_void_p]),
}

_lib = None


def load(path: str | None = None):
    """Loads (once) and returns the ctypes library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or os.environ.get("MATMRI_GB300_LIB", LIB_PATH)
    if not os.path.exists(p):
        raise ImportError(f"libmatmri_gb300.so not found at {p}: run matmri_gb300.build.build() "
                          "(there is no CPU fallback)")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(code: int):
    if code != MMR_OK:
        buf = C.create_string_buffer(1024)
        load().mmr_last_error(buf, 1024)
        raise MatmriError(code, buf.value.decode(errors="replace"))


def check_device_error(stream=None):
    """Raises MatmriError (TIMEOUT) when a bounded device wait ran out since the last check, and
    clears the flag.  For callers that pass device arrays: calls given host arrays check it
    themselves before returning.  `stream`: a cudaStream_t handle (int) or None for the default
    stream; it is synchronised."""
    check(load().mmr_check_device_error(C.c_void_p(stream or 0)))


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))
