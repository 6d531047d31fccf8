"""TEST INFRASTRUCTURE ONLY: Python bindings of the CPU oracle (sw_oracle.cpp,
sw_elastic_oracle.cpp, sw_vd_oracle.cpp).

The oracle is a plain C++ restatement of SeismicWaves.jl's acoustic
constant-density C-PML algorithm, of its variable-density acoustic 2D
(staggered pressure-velocity) C-PML algorithm and of its isotropic elastic 2D
(P-SV) C-PML algorithm (FP64, plus an FP32 instantiation used to study
single-precision error).  Only the test-suite, ``__graft_entry__.smoke``
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
SRCS = [HERE / "sw_oracle.cpp", HERE / "sw_elastic_oracle.cpp", HERE / "sw_vd_oracle.cpp"]
DEPS = SRCS + [HERE / "oracle_common.h"]
LIB = HERE / "_build" / "libsworacle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compile the oracle into oracle/_build/libsworacle.so (g++ -O3 -fopenmp)."""
    LIB.parent.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < max(f.stat().st_mtime for f in DEPS):
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
        cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp)] + [str(f) for f in SRCS]
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
                                                 i, i, P, P, P, P, P, i, i, d]
        lib.oracle_acoustic_gradient.restype = i
        lib.oracle_max_threads.restype = i
        lib.oracle_spread_positions.argtypes = [P, P, i, P, P, i, i, d, P, P, P, ctypes.c_long]
        lib.oracle_spread_positions.restype = ctypes.c_long
        lib.oracle_bessel_i0.argtypes = [d]
        lib.oracle_bessel_i0.restype = d
        lib.oracle_acoustic_forward_snap.argtypes = [i, P, P, d, i, P, P, i, i, P, P, i, P, P, i, i, P]
        lib.oracle_acoustic_forward_snap.restype = i
        lib.oracle_elastic_forward_snap.argtypes = [P, P, d, i, i, P, P, P, i, i, P, i, i, i, P, P, P, P, P, i, P,
                                                    P, P, P, i, i, P]
        lib.oracle_elastic_forward_snap.restype = i
        lib.oracle_interp.argtypes = [P, i, i, i, i, i, P]
        lib.oracle_interp.restype = None
        lib.oracle_back_interp.argtypes = [P, i, i, P, i, i, i, P]
        lib.oracle_back_interp.restype = None
        lib.oracle_elastic_forward.argtypes = [i, P, P, d, i, i, P, P, P, i, i, P, i, i, i, P, P, P, P, P, i, P, P,
                                               P, P, i]
        lib.oracle_elastic_forward.restype = i
        lib.oracle_elastic_gradient.argtypes = [i, P, P, d, i, i, P, P, P, i, i, P, i, i, i, P, P, P, P, P, i, P,
                                                P, P, P, P, i, i, P, i, i, i, P, P, P, P, P, P, P, i, i, d]
        lib.oracle_elastic_gradient.restype = i
        lib.oracle_vd_forward.argtypes = [i, P, P, d, i, P, P, i, P, i, i, P, P, i, P, P, i, i, P]
        lib.oracle_vd_forward.restype = i
        lib.oracle_vd_gradient.argtypes = [i, P, P, d, i, P, P, i, P, i, i, P, P, i, P, P, P, i, i, P, i, i, i, P,
                                           P, P, P, P, P, i, i, d]
        lib.oracle_vd_gradient.restype = i
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
                      f32=False, nthreads=0, ccts_dt=None):
    """swgradient_1shot! (CD) plus calcmisfit for one shot.

    Returns (grad (shape of vp), misfit, traces).  ``invcov`` may be None
    (identity), a 1-D diagonal, or a dense (nt, nt) matrix.  ``ccts_dt``:
    CCTSMisfit(ccts_dt) instead of the L2 misfit.
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
                                         int(nthreads or max_threads()), 0 if ccts_dt is None else 1,
                                         float(ccts_dt or 0.0))
    if rc != 0:
        raise RuntimeError(f"oracle_acoustic_gradient failed ({rc})")
    return grad, float(misfit[0]), traces


# ---------------------------------------------------------------------------
# elastic 2D
# ---------------------------------------------------------------------------
def bessel_i0(x: float) -> float:
    return load().oracle_bessel_i0(float(x))


def interp(m, dims, method=0):
    """interp(method, m, dims) for a 2-D array (interpolations.jl:1-43); dims subset of (1, 2)."""
    m = np.asfortranarray(m, dtype=np.float64)
    nx, nz = m.shape
    di, dj = int(1 in dims), int(2 in dims)
    out = np.zeros((nx - di, nz - dj), dtype=np.float64, order="F")
    load().oracle_interp(_p(m), nx, nz, di, dj, int(method), _p(out))
    return out


def back_interp(m, g, dims, method=0):
    """back_interp(method, m, g, dims) for 2-D arrays (interpolations.jl:15-28)."""
    m = np.asfortranarray(m, dtype=np.float64)
    g = np.asfortranarray(g, dtype=np.float64)
    nx, nz = m.shape
    res = np.zeros((nx, nz), dtype=np.float64, order="F")
    load().oracle_back_interp(_p(m), nx, nz, _p(g), int(1 in dims), int(2 in dims), int(method), _p(res))
    return res


def spread_positions(n, h, positions, shift=(0.0, 0.0), mirror=False, r=4, beta=6.31):
    """spread_positions (utils.jl:168-214, free surface on the grid bound).

    Returns one (ij (npts, 2) int32 1-based, coef (npts,) float64) pair per position.
    """
    pos = np.asfortranarray(positions, dtype=np.float64)
    npos = pos.shape[0]
    nn = np.array(n, dtype=np.int32)
    hh = np.array(h, dtype=np.float64)
    sh = np.array(shift, dtype=np.float64)
    lib = load()
    tot = lib.oracle_spread_positions(_p(nn), _p(hh), npos, _p(pos), _p(sh), int(bool(mirror)), int(r),
                                      float(beta), None, None, None, 0)
    cnt = np.zeros(npos, dtype=np.int32)
    ij = np.zeros((max(tot, 1), 2), dtype=np.int32)
    coef = np.zeros(max(tot, 1), dtype=np.float64)
    lib.oracle_spread_positions(_p(nn), _p(hh), npos, _p(pos), _p(sh), int(bool(mirror)), int(r), float(beta),
                                _p(cnt), _p(ij), _p(coef), int(tot))
    out, q = [], 0
    for c in cnt:
        out.append((ij[q:q + c].copy(), coef[q:q + c].copy()))
        q += c
    return out


def _pack(tables, nitems):
    """[table0 (list per item), table1] -> cnt, ij, coef in the oracle's packing."""
    cnt = np.zeros(2 * nitems, dtype=np.int32)
    ijs, cs = [], []
    for t in range(2):
        assert len(tables[t]) == nitems
        for k, (ij, c) in enumerate(tables[t]):
            cnt[t * nitems + k] = len(c)
            ijs.append(np.asarray(ij, dtype=np.int32).reshape(-1, 2))
            cs.append(np.asarray(c, dtype=np.float64).reshape(-1))
    ij = np.ascontiguousarray(np.concatenate(ijs) if ijs else np.zeros((1, 2)), dtype=np.int32)
    coef = np.ascontiguousarray(np.concatenate(cs) if cs else np.zeros(1), dtype=np.float64)
    if ij.size == 0:
        ij, coef = np.zeros((1, 2), np.int32), np.zeros(1)
    return cnt, ij, coef


def _elastic_common(lam, mu, rho, h, cpml, shot):
    lam = np.asfortranarray(lam, dtype=np.float64)
    mu = np.asfortranarray(mu, dtype=np.float64)
    rho = np.asfortranarray(rho, dtype=np.float64)
    n = np.array(lam.shape, dtype=np.int32)
    hh = np.array(h, dtype=np.float64)
    kind = 0 if shot["kind"] == "mt" else 1
    tf = np.asfortranarray(shot["srctf"], dtype=np.float64)
    nt = tf.shape[0]
    nsrc = tf.shape[-1]
    mt = np.ascontiguousarray(shot.get("momtens", np.zeros((nsrc, 3))), dtype=np.float64).reshape(nsrc, 3)
    sc, sij, scoef = _pack(shot["src_tables"], nsrc)
    nrec = len(shot["rec_tables"][0])
    rc_, rij, rcoef = _pack(shot["rec_tables"], nrec)
    cp = np.ascontiguousarray(cpml, dtype=np.float64)
    return lam, mu, rho, n, hh, kind, tf, nt, nsrc, mt, sc, sij, scoef, nrec, rc_, rij, rcoef, cp


def elastic_forward(lam, mu, rho, h, dt, halo, freetop, cpml, shot, *, interp_rho=0, interp_mu=0, f32=False,
                    nthreads=0):
    """swforward_1shot! (elastic 2D).  ``shot``: dict(kind="mt"|"force", srctf
    ((nt, nsrc) or (nt, 2, nsrc), already divided by dx*dz), momtens (nsrc, 3)
    [Mxx, Mzz, Mxz], src_tables [table0, table1], rec_tables [ux, uz]), each
    table a list of (ij, coef) per position.  Returns traces (nt, 2, nrec)."""
    (lam, mu, rho, n, hh, kind, tf, nt, nsrc, mt, sc, sij, scoef, nrec, rcn, rij, rcoef,
     cp) = _elastic_common(lam, mu, rho, h, cpml, shot)
    traces = np.zeros((nt, 2, nrec), dtype=np.float64, order="F")
    rc = load().oracle_elastic_forward(int(f32), _p(n), _p(hh), float(dt), int(halo), int(bool(freetop)),
                                       _p(lam), _p(mu), _p(rho), int(interp_rho), int(interp_mu), _p(cp), nt,
                                       kind, nsrc, _p(tf), _p(mt), _p(sc), _p(sij), _p(scoef), nrec, _p(rcn),
                                       _p(rij), _p(rcoef), _p(traces), int(nthreads or max_threads()))
    if rc != 0:
        raise RuntimeError(f"oracle_elastic_forward failed ({rc})")
    return traces


def elastic_gradient(lam, mu, rho, h, dt, halo, freetop, cpml, shot, observed, *, invcov=None, windows=(),
                     check_freq=1, mute_src=0, mute_rec=0, src_pos=None, rec_pos=None, interp_rho=0,
                     interp_mu=0, f32=False, nthreads=0, ccts_dt=None):
    """swgradient_1shot! (elastic 2D) plus calcmisfit.  Returns
    (dict(rho=, lambda=, mu=) float64 (nx, nz), misfit, traces (nt, 2, nrec)).
    ``ccts_dt``: CCTSMisfit(ccts_dt) per component trace instead of the L2 misfit."""
    (lam, mu, rho, n, hh, kind, tf, nt, nsrc, mt, sc, sij, scoef, nrec, rcn, rij, rcoef,
     cp) = _elastic_common(lam, mu, rho, h, cpml, shot)
    observed = np.asfortranarray(observed, dtype=np.float64)
    assert observed.shape == (nt, 2, nrec)
    if invcov is None:
        ikind, ic = 0, np.zeros(1)
    else:
        ic = np.asfortranarray(invcov, dtype=np.float64)
        ikind = 1 if ic.ndim == 1 else 2
    win = np.array(list(windows), dtype=np.int32).reshape(-1)
    nwin = len(win) // 2
    if win.size == 0:
        win = np.zeros(2, dtype=np.int32)
    sp = np.asfortranarray(src_pos if src_pos is not None else np.zeros((nsrc, 2)), dtype=np.float64)
    rp = np.asfortranarray(rec_pos if rec_pos is not None else np.zeros((nrec, 2)), dtype=np.float64)
    traces = np.zeros((nt, 2, nrec), dtype=np.float64, order="F")
    g = {k: np.zeros(lam.shape, dtype=np.float64, order="F") for k in ("rho", "lambda", "mu")}
    misfit = np.zeros(1, dtype=np.float64)
    rc = load().oracle_elastic_gradient(int(f32), _p(n), _p(hh), float(dt), int(halo), int(bool(freetop)),
                                        _p(lam), _p(mu), _p(rho), int(interp_rho), int(interp_mu), _p(cp), nt,
                                        kind, nsrc, _p(tf), _p(mt), _p(sc), _p(sij), _p(scoef), nrec, _p(rcn),
                                        _p(rij), _p(rcoef), _p(observed), _p(ic), ikind, nwin, _p(win),
                                        int(check_freq), int(mute_src), int(mute_rec), _p(sp), _p(rp),
                                        _p(traces), _p(g["rho"]), _p(g["lambda"]), _p(g["mu"]), _p(misfit),
                                        int(nthreads or max_threads()), 0 if ccts_dt is None else 1,
                                        float(ccts_dt or 0.0))
    if rc != 0:
        raise RuntimeError(f"oracle_elastic_gradient failed ({rc})")
    return g, float(misfit[0]), traces


def acoustic_forward_snapshots(vp, h, dt, halo, cpml, srctf, src_idx, rec_idx, snapevery, *, nthreads=0):
    """swforward_1shot! with a LinearSnapshotter: (traces, snapshots (nsnap, *vp.shape))."""
    vp = np.asfortranarray(vp, dtype=np.float64)
    N, n, hh = _grid(vp, h)
    srctf = np.asfortranarray(srctf, dtype=np.float64)
    nt, nsrc = srctf.shape
    src_idx = np.asfortranarray(src_idx, dtype=np.int32)
    rec_idx = np.asfortranarray(rec_idx, dtype=np.int32)
    nrec = rec_idx.shape[0]
    cpml = np.ascontiguousarray(cpml, dtype=np.float64)
    traces = np.zeros((nt, nrec), dtype=np.float64, order="F")
    nsnap = nt // snapevery
    snaps = np.zeros((nsnap, vp.size), dtype=np.float64)
    rc = load().oracle_acoustic_forward_snap(N, _p(n), _p(hh), float(dt), int(halo), _p(vp), _p(cpml), nt, nsrc,
                                             _p(src_idx), _p(srctf), nrec, _p(rec_idx), _p(traces),
                                             int(nthreads or max_threads()), int(snapevery), _p(snaps))
    if rc != 0:
        raise RuntimeError(f"oracle_acoustic_forward_snap failed ({rc})")
    return traces, np.stack([s.reshape(vp.shape, order="F") for s in snaps]) if nsnap else snaps


def elastic_forward_snapshots(lam, mu, rho, h, dt, halo, freetop, cpml, shot, snapevery, *, interp_rho=0,
                              interp_mu=0, nthreads=0):
    """Elastic swforward_1shot! with snapshots: (traces, blocks (nsnap, B)) with B the
    concatenated ux, uz, sxx, szz, sxz fields (column-major)."""
    (lam, mu, rho, n, hh, kind, tf, nt, nsrc, mt, sc, sij, scoef, nrec, rcn, rij, rcoef,
     cp) = _elastic_common(lam, mu, rho, h, cpml, shot)
    nx, nz = lam.shape
    B = (nx - 1) * nz + nx * (nz - 1) + 2 * nx * nz + (nx - 1) * (nz - 1)
    traces = np.zeros((nt, 2, nrec), dtype=np.float64, order="F")
    snaps = np.zeros((nt // snapevery, B), dtype=np.float64)
    rc = load().oracle_elastic_forward_snap(_p(n), _p(hh), float(dt), int(halo), int(bool(freetop)), _p(lam),
                                            _p(mu), _p(rho), int(interp_rho), int(interp_mu), _p(cp), nt, kind,
                                            nsrc, _p(tf), _p(mt), _p(sc), _p(sij), _p(scoef), nrec, _p(rcn), _p(rij),
                                            _p(rcoef), _p(traces), int(nthreads or max_threads()), int(snapevery),
                                            _p(snaps))
    if rc != 0:
        raise RuntimeError(f"oracle_elastic_forward_snap failed ({rc})")
    return traces, snaps


# ---------------------------------------------------------------------------
# variable-density acoustic 2D
# ---------------------------------------------------------------------------
def _vd_common(vp, rho, h, cpml, srctf, src_idx, rec_idx):
    vp = np.asfortranarray(vp, dtype=np.float64)
    rho = np.asfortranarray(rho, dtype=np.float64)
    assert vp.ndim == 2 and vp.shape == rho.shape
    n = np.array(vp.shape, dtype=np.int32)
    hh = np.array(h[:2], dtype=np.float64)
    srctf = np.asfortranarray(srctf, dtype=np.float64)
    src_idx = np.asfortranarray(src_idx, dtype=np.int32)
    rec_idx = np.asfortranarray(rec_idx, dtype=np.int32)
    cpml = np.ascontiguousarray(cpml, dtype=np.float64)
    return vp, rho, n, hh, srctf, src_idx, rec_idx, cpml


def vd_forward(vp, rho, h, dt, halo, cpml, srctf, src_idx, rec_idx, *, interp=0, f32=False, nthreads=0,
               snapevery=0):
    """swforward_1shot! of AcousticVDStaggeredCPMLWaveSimulation (2D) for one shot.

    ``srctf`` (nt, nsrc) is already scaled by dt vp(src)^2 rho(src) / (dx dz).
    Returns traces (nt, nrec); with ``snapevery`` > 0 also a list of
    (p, vx, vz) snapshots after the steps it = snapevery, 2 snapevery, ...
    """
    vp, rho, n, hh, srctf, src_idx, rec_idx, cpml = _vd_common(vp, rho, h, cpml, srctf, src_idx, rec_idx)
    nt, nsrc = srctf.shape
    nrec = rec_idx.shape[0]
    nx, nz = vp.shape
    traces = np.zeros((nt, nrec), dtype=np.float64, order="F")
    B = nx * nz + (nx - 1) * nz + nx * (nz - 1)
    nsnap = nt // snapevery if snapevery > 0 else 0
    snaps = np.zeros(max(nsnap, 1) * B, dtype=np.float64)
    rc = load().oracle_vd_forward(int(f32), _p(n), _p(hh), float(dt), int(halo), _p(vp), _p(rho), int(interp),
                                  _p(cpml), nt, nsrc, _p(src_idx), _p(srctf), nrec, _p(rec_idx), _p(traces),
                                  int(nthreads or max_threads()), int(snapevery), _p(snaps))
    if rc != 0:
        raise RuntimeError(f"oracle_vd_forward failed ({rc})")
    if snapevery <= 0:
        return traces
    out = []
    for k in range(nsnap):
        b = snaps[k * B:(k + 1) * B]
        p = b[:nx * nz].reshape((nx, nz), order="F")
        vx = b[nx * nz:nx * nz + (nx - 1) * nz].reshape((nx - 1, nz), order="F")
        vz = b[nx * nz + (nx - 1) * nz:].reshape((nx, nz - 1), order="F")
        out.append((p, vx, vz))
    return traces, out


def vd_gradient(vp, rho, h, dt, halo, cpml, srctf, src_idx, rec_idx, observed, *, interp=0, invcov=None,
                windows=(), check_freq=1, mute_src=0, mute_rec=0, src_pos=None, rec_pos=None, f32=False,
                nthreads=0, ccts_dt=None):
    """swgradient_1shot! of the VD simulation plus calcmisfit for one shot.

    Returns ({"vp": ..., "rho": ...}, misfit, traces).  ``ccts_dt``: CCTSMisfit(ccts_dt).
    """
    vp, rho, n, hh, srctf, src_idx, rec_idx, cpml = _vd_common(vp, rho, h, cpml, srctf, src_idx, rec_idx)
    nt, nsrc = srctf.shape
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
    sp = np.asfortranarray(src_pos if src_pos is not None else np.zeros((nsrc, 2)), dtype=np.float64)
    rp = np.asfortranarray(rec_pos if rec_pos is not None else np.zeros((nrec, 2)), dtype=np.float64)
    traces = np.zeros((nt, nrec), dtype=np.float64, order="F")
    gvp = np.zeros(vp.shape, dtype=np.float64, order="F")
    grho = np.zeros(vp.shape, dtype=np.float64, order="F")
    misfit = np.zeros(1, dtype=np.float64)
    rc = load().oracle_vd_gradient(int(f32), _p(n), _p(hh), float(dt), int(halo), _p(vp), _p(rho), int(interp),
                                   _p(cpml), nt, nsrc, _p(src_idx), _p(srctf), nrec, _p(rec_idx), _p(observed),
                                   _p(ic), kind, nwin, _p(win), int(check_freq), int(mute_src), int(mute_rec),
                                   _p(sp), _p(rp), _p(traces), _p(gvp), _p(grho), _p(misfit),
                                   int(nthreads or max_threads()), 0 if ccts_dt is None else 1,
                                   float(ccts_dt or 0.0))
    if rc != 0:
        raise RuntimeError(f"oracle_vd_gradient failed ({rc})")
    return {"vp": gvp, "rho": grho}, float(misfit[0]), traces
