"""Tile/kernel autotuner for the stencil launches.

For a given simulation and batch of shots, times a short batched forward
(the first `steps` time steps of every shot) for each candidate of the 2D
stencil implementation (register-pipelined with 4, 8 or 16 warps per block,
rows staged through shared memory by cp.async, or the TMA pipeline) and band
height, and installs the fastest with
sw_wavesim_set_tuning.  Results are cached per (grid, halo, number of shots).
The numerics do not depend on the choice (all candidates run the same
arithmetic), so tuning never changes results.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib

_cache: dict = {}

CANDIDATES_2D = [(0, 4), (0, 8), (0, 16), (2, 8), (512, 8), (1, 32), (1, 64)]
CANDIDATES_3D = [(0, 8), (0, 16), (0, 32), (0, 64)]


def autotune(ctx: _lib.Context, ws_handle, grid_key, shots_structs, nshots: int, ndim: int, steps: int = 24,
             on_device: int = 0):
    """Pick and install (variant, tz) for `ws_handle`; returns the choice and the timings.

    `shots_structs` is a ctypes array of SwAcousticShot; their nt is capped at
    `steps` for the trial runs (the caller's arrays are only read, traces are
    overwritten).
    """
    key = (grid_key, nshots, ndim)
    lib = ctx.lib
    if key in _cache:
        v, tz = _cache[key][0]
        ctx.check(lib.sw_wavesim_set_tuning(ws_handle, tz, v), "sw_wavesim_set_tuning")
        return _cache[key]
    saved = [s.nt for s in shots_structs]
    for s in shots_structs:
        s.nt = min(s.nt, steps)
    timings = {}
    try:
        for v, tz in (CANDIDATES_2D if ndim == 2 else CANDIDATES_3D):
            ctx.check(lib.sw_wavesim_set_tuning(ws_handle, tz, v), "sw_wavesim_set_tuning")
            ctx.check(lib.sw_acoustic_forward(ws_handle, nshots, shots_structs, on_device), "tuning forward")
            best = float("inf")
            for _ in range(2):
                t0 = time.perf_counter()
                ctx.check(lib.sw_acoustic_forward(ws_handle, nshots, shots_structs, on_device), "tuning forward")
                best = min(best, time.perf_counter() - t0)
            timings[(v, tz)] = best
    finally:
        for s, nt in zip(shots_structs, saved):
            s.nt = nt
    choice = min(timings, key=timings.get)
    ctx.check(lib.sw_wavesim_set_tuning(ws_handle, choice[1], choice[0]), "sw_wavesim_set_tuning")
    _cache[key] = (choice, timings)
    return _cache[key]
