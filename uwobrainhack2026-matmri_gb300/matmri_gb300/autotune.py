"""Autotuner for the SENSE normal operator's launch shapes.

Knobs (``mmr_tuning``): coils per pipeline pass (``coil_chunk``, the grids of
one pass stay resident in L2), gridding tile side (``tile``), coils per CTA in
the gridding kernels (``coil_group``), samples per gridding work item
(``item``) and transform lines per CTA in the FFT passes (``fft_lines``).

The search is a coordinate descent per gridding mode (fused interpolate /
spread, or the precomputed stencil): from the current setting with that mode,
each other knob in turn is swept over its candidates with the rest fixed, for
two rounds, then tile side and coils per CTA jointly (they share the shared
memory); the faster mode's optimum wins.  (One descent over all knobs can
stall in the slower mode: its optimum for the other knobs differs.)
Every candidate is applied once untimed, then timed end to end with CUDA
events around back-to-back normal operators (``mmr_sense_normal``), best of
three.  Results are cached per size class (image
size, oversampled grid, samples, coils, kernel width) and device in a JSON
file (``$MATMRI_GB300_TUNE_CACHE`` or ``~/.cache/matmri_gb300/tuning.json``).
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import _lib

SPACE = {
    "coil_chunk": [4, 8, 16, 32],
    "tile": [16, 32, 64],
    "coil_group": [2, 4, 8],
    "item": [32, 64, 128, 256],
    "fft_lines": [4, 8, 16],
    "normal_mode": [1, 2],
}
ORDER = ["normal_mode", "item", "coil_group", "tile", "fft_lines", "coil_chunk"]


def _cache_path():
    p = os.environ.get("MATMRI_GB300_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "matmri_gb300", "tuning.json")


def _device_key():
    lib = _lib.load()
    sm, smem, ma, mi = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    _lib.check(lib.mmr_device_info(C.byref(sm), C.byref(smem), C.byref(ma), C.byref(mi)))
    return f"sm{ma.value}{mi.value}x{sm.value}"


def size_class(op) -> str:
    S = op.S
    osN = getattr(S, "osN", None)
    kw = getattr(S, "kwidth", 0)
    return f"N{'x'.join(map(str, op.imN))}_G{'x'.join(map(str, osN or []))}_M{op.M}_C{op.C}_W{kw}"


def time_normal(op, x_ptr, y_ptr, reps=5, trials=3) -> float:
    """ms of one normal operator application: CUDA events around `reps` back-to-back applications on
    the current stream after one untimed application (which builds anything a setting needs first),
    best of `trials`.  End to end, so per-kernel launch gaps count as they do in a solve."""
    import torch
    lib = _lib.load()
    st = torch.cuda.current_stream()
    sp = st.cuda_stream
    _lib.check(lib.mmr_sense_normal(op.handle, x_ptr, y_ptr, sp))
    best = float("inf")
    for _ in range(trials):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            _lib.check(lib.mmr_sense_normal(op.handle, x_ptr, y_ptr, sp))
        e1.record(st)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / reps)
    return best


KNOBS = ["coil_chunk", "tile", "coil_group", "item", "fft_lines", "normal_mode"]


def search(op, measure, rounds=2, verbose=False):
    """The search itself: ``measure()`` times the normal operator of ``op`` at its current setting
    (ms).  Returns (knobs, ms) of the fastest setting found and leaves ``op`` set to it."""
    start = dict(zip(KNOBS, op.get_tuning()))

    def timed(trial):
        op.set_tuning(**trial)
        t = measure()
        if verbose:
            print(f"autotune {trial} -> {t:.4f} ms")
        return t

    best_t, best = float("inf"), None
    for mode in SPACE["normal_mode"]:
        cur = dict(start, normal_mode=mode)
        cur_t = timed(cur)
        for _ in range(rounds):
            for knob in ORDER:
                if knob == "normal_mode":
                    continue
                for v in SPACE[knob]:
                    if v == cur[knob] or (knob == "coil_chunk" and v > op.C):
                        continue
                    trial = dict(cur, **{knob: v})
                    t = timed(trial)
                    if t < cur_t:
                        cur_t, cur = t, trial
        # tile side and coils per CTA trade shared memory against each other: sweep them jointly
        for tile in SPACE["tile"]:
            for cgrp in SPACE["coil_group"]:
                if (tile, cgrp) == (cur["tile"], cur["coil_group"]):
                    continue
                trial = dict(cur, tile=tile, coil_group=cgrp)
                t = timed(trial)
                if t < cur_t:
                    cur_t, cur = t, trial
        if cur_t < best_t:
            best_t, best = cur_t, cur
    op.set_tuning(**best)
    return best, best_t


def autotune(op, reps=5, rounds=2, use_cache=True, verbose=False) -> dict:
    """Tunes ``op`` (an mrSampOp over a 2D nufftOp) in place; returns the chosen knobs."""
    key = f"{_device_key()}/{size_class(op)}"
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except Exception:
            cache = {}
    if use_cache and key in cache:
        op.set_tuning(**cache[key]["tuning"])
        return dict(cache[key]["tuning"])
    import torch  # device buffers for the probe
    n = int(np.prod(op.imN))
    x = torch.randn(n, dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    cur, best_t = search(op, lambda: time_normal(op, x.data_ptr(), y.data_ptr(), reps), rounds, verbose)
    if use_cache:
        cache[key] = {"tuning": cur, "normal_ms": best_t}
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, path)
    return cur
