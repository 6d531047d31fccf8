"""Tile/kernel autotuner for the stencil launches.

For a given simulation and batch of shots it times short trial runs of each
candidate stencil configuration and installs the fastest with
sw_wavesim_set_tuning.  Trials are short batched *gradients* (forward with
checkpoints, misfit, adjoint with recompute) when the caller hands gradient
outputs and the trial record can hold two checkpoint periods -- so the
forward, recompute and adjoint kinds all weigh in, each with its own time
read from the library's per-kind event timing -- and short forwards
otherwise (3D, where gradient trials would be long).  Candidates for 2D: the
register-pipelined stencil with 4-, 8- or 16-row bands and with 8 warps per
block, the cp.async-staged stencil, two time steps per launch, and the
grouped adjoint; for 3D the band height, 8 y rows per block, the inner
rows without the software pipeline and the single-launch step.  A second
stage then picks the band height of the forward, recompute and adjoint
stencils separately, each from its own per-kind time
(sw_wavesim_set_band_heights).  Results are cached per (grid, halo, shots,
dimension, gradient or forward trials).  The numerics do not depend on the
choice (every candidate runs the same rounded arithmetic), so tuning never
changes results.

autotune_tz does the same for the variable-density and elastic simulations,
whose only knob is the band height (sw_acoustic_vd_set_tuning /
sw_elastic_set_tuning).
"""
from __future__ import annotations

import time

from . import _lib

_cache: dict = {}

# (variant, tz) of sw_wavesim_set_tuning; 2D: 262144 = the x strips in the
# main blocks' per-point path instead of extra blocks of their own
CANDIDATES_2D = [(0, 4), (0, 8), (0, 16), (2, 8), (512, 8), (1024, 0), (256, 8), (262144, 8)]
# 3D: 131072 = inner rows without the software pipeline, 65536 = one launch per step
CANDIDATES_3D = [(0, 8), (0, 16), (0, 32), (2, 8), (131072, 8), (131072, 16), (131074, 16), (65536, 16)]
KIND_NAMES = {0: "forward", 4: "recompute", 1: "adjoint"}
# band heights tried per stencil kind after the variant is chosen (2D gradients)
TZ_KIND_2D = (4, 8, 16)


def _kind_ms(ctx):
    return {name: ctx.profile_read(k)[0] for k, name in KIND_NAMES.items()}


def _best_of(trial, n=2):
    best = float("inf")
    for _ in range(n):
        t0 = time.perf_counter()
        trial()
        best = min(best, time.perf_counter() - t0)
    return best


def autotune(ctx: _lib.Context, ws_handle, grid_key, shots_structs, nshots: int, ndim: int, steps: int = 24,
             on_device: int = 0, gradient_out=None, check_freq: int = 0, candidates=None, kind_tz=TZ_KIND_2D):
    """Pick and install the stencil configuration of `ws_handle`; returns a dict

    variant, tz        -- the sw_wavesim_set_tuning arguments installed
    band_heights       -- (forward, recompute, adjoint) of sw_wavesim_set_band_heights, or None
    trial_s            -- {(variant, tz): best seconds of a trial}
    per_kind_ms        -- {(variant, tz): {kind: ms}} (gradient trials only)
    band_ms            -- {tz: {kind: ms}} of the per-kind stage (or {})

    `shots_structs` is a ctypes array of SwAcousticShot; their nt is capped for
    the trial runs (the caller's arrays are only read, traces are
    overwritten).  With `gradient_out` = (grad pointer, misfit pointer) and the
    simulation's checkpoint period `check_freq`, trials are gradients of
    max(steps, 2 check_freq + 2) steps.  Then, for a one-step 2D winner, each
    band height of `kind_tz` is run once more with the per-kind event timing,
    every kind takes the band that was fastest for it, and the mixed
    configuration is kept if a timed trial confirms it is not slower.
    """
    key = (grid_key, nshots, ndim, gradient_out is not None)
    lib = ctx.lib

    def install(v, tz, bands):
        ctx.check(lib.sw_wavesim_set_tuning(ws_handle, tz, v), "sw_wavesim_set_tuning")
        b = bands or (0, 0, 0)
        ctx.check(lib.sw_wavesim_set_band_heights(ws_handle, *b), "sw_wavesim_set_band_heights")

    if key in _cache:
        r = _cache[key]
        install(r["variant"], r["tz"], r["band_heights"])
        return r
    grad = gradient_out is not None
    cap = max(steps, 2 * check_freq + 2) if grad else steps
    saved = [s.nt for s in shots_structs]
    for s in shots_structs:
        s.nt = min(s.nt, cap)
    if grad and any(s.nt <= check_freq for s in shots_structs):
        grad = False  # records too short for a checkpointed trial: time forwards instead
        for s, nt in zip(shots_structs, saved):
            s.nt = min(nt, steps)

    def trial():
        if grad:
            ctx.check(lib.sw_acoustic_gradient(ws_handle, nshots, shots_structs, on_device, gradient_out[0],
                                               gradient_out[1]), "tuning gradient")
        else:
            ctx.check(lib.sw_acoustic_forward(ws_handle, nshots, shots_structs, on_device), "tuning forward")

    def profiled():
        ctx.profile(True)
        try:
            trial()
        finally:
            ctx.profile(False)
        return _kind_ms(ctx)

    timings, per_kind, band_ms = {}, {}, {}
    bands = None
    try:
        for v, tz in (candidates or (CANDIDATES_2D if ndim == 2 else CANDIDATES_3D)):
            install(v, tz, None)
            trial()
            timings[(v, tz)] = _best_of(trial)
            if grad:
                per_kind[(v, tz)] = profiled()
        choice = min(timings, key=timings.get)
        if grad and ndim == 2 and not (choice[0] & 1024) and kind_tz:
            for tz in kind_tz:
                install(choice[0], tz, None)
                trial()
                band_ms[tz] = profiled()
            mixed = tuple(min(band_ms, key=lambda t: band_ms[t][k]) for k in ("forward", "recompute", "adjoint"))
            install(choice[0], 0, mixed)
            trial()
            t_mixed = _best_of(trial)
            timings[("bands",) + mixed] = t_mixed
            if t_mixed <= timings[choice]:
                bands = mixed
    finally:
        for s, nt in zip(shots_structs, saved):
            s.nt = nt
    r = {"variant": choice[0], "tz": 0 if bands else choice[1], "band_heights": bands, "trial_s": timings,
         "per_kind_ms": per_kind, "band_ms": band_ms}
    install(r["variant"], r["tz"], bands)
    _cache[key] = r
    return r


def autotune_tz(key, set_tuning, trial, candidates=(8, 16, 32)):
    """Band height of a variable-density or elastic simulation: `set_tuning(tz)`
    installs a candidate, `trial()` runs one short batched call; the fastest
    of two timed trials per candidate is kept.  Returns (tz, timings)."""
    if key in _cache:
        set_tuning(_cache[key][0])
        return _cache[key]
    timings = {}
    for tz in candidates:
        set_tuning(tz)
        trial()
        timings[tz] = _best_of(trial)
    choice = min(timings, key=timings.get)
    set_tuning(choice)
    _cache[key] = (choice, timings)
    return _cache[key]
