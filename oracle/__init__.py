"""TEST INFRASTRUCTURE ONLY: Python bindings of the CPU oracle (sw_oracle.cpp).

The oracle is a plain C++ restatement of SeismicWaves.jl's acoustic
constant-density C-PML algorithm (FP64, plus an FP32 instantiation used to
study single-precision error).  Only the test-suite, ``__graft_entry__.smoke``
and the CPU-baseline leg of ``bench.py`` may import this module; the product
(``seismicwaves.jl_gb300``) never does.

Array conventions follow the reference (Julia, column-major): grids are numpy
arrays of shape ``(nx, nz)`` or ``(nx, ny, nz)`` in Fortran order, traces are
``(nt, nrec)``, positions ``(npos, ndim)``, grid indices are 1-based.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "sw_oracle.cpp"
LIB = HERE / "_build" / "libsworacle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compile the oracle into oracle/_build/libsworacle.so (g++ -O3 -fopenmp)."""
    LIB.parent.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
        cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(SRC)]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(str(LIB))
        d, i = ctypes.c_double, ctypes.c_int
        P = ctypes.c_void_p
        lib.oracle_cpml_axis.argtypes = [d, d, i, d, d, d, i, P]
        lib.oracle_cpml_axis.restype = None
        lib.oracle_acoustic_forward.argtypes = [i, i, P, P, d, i, P, P, i, i, P, P, i, P, P, i]
        lib.oracle_acoustic_forward.restype = i
        lib.oracle_acoustic_gradient.argtypes = [i, i, P, P, d, i, P, P, i, i, P, P, i, P, P, P, i, i, P, i,
                                                 i, i, P, P, P, P, P, i]
        lib.oracle_acoustic_gradient.restype = i
        lib.oracle_max_threads.restype = i
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def max_threads() -> int:
    return load().oracle_max_threads()


def cpml_block(vel_max, dt, halo, rcoef, h, f0, freetop_axis):
    """One axis of C-PML coefficients packed as [a, a_h, b, b_h] (float64)."""
    n = 2 * (2 * (halo + 1)) + 2 * (2 * halo)
    out = np.zeros(n, dtype=np.float64)
    load().oracle_cpml_axis(float(vel_max), float(dt), int(halo), float(rcoef), float(h), float(f0),
                            int(bool(freetop_axis)), _p(out))
    return out


def cpml_blocks(vp, h, dt, halo, rcoef, f0, freetop, vel_max=None):
    """init_bdc! for all axes, concatenated (axis 0 first)."""
    vmax = float(np.max(vp)) if vel_max is None else float(vel_max)
    N = vp.ndim
    return np.concatenate([cpml_block(vmax, dt, halo, rcoef, h[d], f0, freetop and d == N - 1)
                           for d in range(N)])


def _grid(vp, h):
    N = vp.ndim
    n = np.array(list(vp.shape) + [1] * (3 - N), dtype=np.int32)
    hh = np.array(list(h) + [1.0] * (3 - N), dtype=np.float64)
    return N, n, hh


def acoustic_forward(vp, h, dt, halo, cpml, srctf, src_idx, rec_idx, *, f32=False, nthreads=0):
    """swforward_1shot! for one shot; returns traces (nt, nrec) float64."""
    vp = np.asfortranarray(vp, dtype=np.float64)
    N, n, hh = _grid(vp, h)
    srctf = np.asfortranarray(srctf, dtype=np.float64)
    nt, nsrc = srctf.shape
    src_idx = np.asfortranarray(src_idx, dtype=np.int32)
    rec_idx = np.asfortranarray(rec_idx, dtype=np.int32)
    nrec = rec_idx.shape[0]
    cpml = np.ascontiguousarray(cpml, dtype=np.float64)
    traces = np.zeros((nt, nrec), dtype=np.float64, order="F")
    rc = load().oracle_acoustic_forward(int(f32), N, _p(n), _p(hh), float(dt), int(halo), _p(vp), _p(cpml),
                                        nt, nsrc, _p(src_idx), _p(srctf), nrec, _p(rec_idx), _p(traces),
                                        int(nthreads or max_threads()))
    if rc != 0:
        raise RuntimeError(f"oracle_acoustic_forward failed ({rc})")
    return traces


def acoustic_gradient(vp, h, dt, halo, cpml, srctf, src_idx, rec_idx, observed, *, invcov=None,
                      windows=(), check_freq=1, mute_src=0, mute_rec=0, src_pos=None, rec_pos=None,
                      f32=False, nthreads=0):
    """swgradient_1shot! (CD) plus calcmisfit for one shot.

    Returns (grad (shape of vp), misfit, traces).  ``invcov`` may be None
    (identity), a 1-D diagonal, or a dense (nt, nt) matrix.
    """
    vp = np.asfortranarray(vp, dtype=np.float64)
    N, n, hh = _grid(vp, h)
    srctf = np.asfortranarray(srctf, dtype=np.float64)
    nt, nsrc = srctf.shape
    src_idx = np.asfortranarray(src_idx, dtype=np.int32)
    rec_idx = np.asfortranarray(rec_idx, dtype=np.int32)
    nrec = rec_idx.shape[0]
    observed = np.asfortranarray(observed, dtype=np.float64)
    assert observed.shape == (nt, nrec)
    if invcov is None:
        kind, ic = 0, np.zeros(1)
    else:
        ic = np.asfortranarray(invcov, dtype=np.float64)
        kind = 1 if ic.ndim == 1 else 2
    win = np.array(list(windows), dtype=np.int32).reshape(-1)
    nwin = len(win) // 2
    if win.size == 0:
        win = np.zeros(2, dtype=np.int32)
    sp = np.asfortranarray(src_pos if src_pos is not None else np.zeros((nsrc, N)), dtype=np.float64)
    rp = np.asfortranarray(rec_pos if rec_pos is not None else np.zeros((nrec, N)), dtype=np.float64)
    cpml = np.ascontiguousarray(cpml, dtype=np.float64)
    traces = np.zeros((nt, nrec), dtype=np.float64, order="F")
    grad = np.zeros(vp.shape, dtype=np.float64, order="F")
    misfit = np.zeros(1, dtype=np.float64)
    rc = load().oracle_acoustic_gradient(int(f32), N, _p(n), _p(hh), float(dt), int(halo), _p(vp), _p(cpml),
                                         nt, nsrc, _p(src_idx), _p(srctf), nrec, _p(rec_idx), _p(observed),
                                         _p(ic), kind, nwin, _p(win), int(check_freq), int(mute_src),
                                         int(mute_rec), _p(sp), _p(rp), _p(traces), _p(grad), _p(misfit),
                                         int(nthreads or max_threads()))
    if rc != 0:
        raise RuntimeError(f"oracle_acoustic_gradient failed ({rc})")
    return grad, float(misfit[0]), traces
