"""Shared builders for the parity tests: seeded synthetic models and shots,
and thin drivers that run one case through the GPU library (C ABI) and
through the CPU oracle with identical inputs."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Shot:
    src_pos: np.ndarray            # (nsrc, ndim) metres
    rec_pos: np.ndarray            # (nrec, ndim) metres
    tf: np.ndarray                 # (nt, nsrc) unscaled source time functions
    f0: float
    nt: int
    observed: np.ndarray | None = None
    invcov: np.ndarray | None = None
    windows: list = field(default_factory=list)


@dataclass
class Case:
    vp: np.ndarray                 # Fortran-ordered (nx, nz) or (nx, ny, nz)
    h: tuple
    dt: float
    halo: int
    freetop: bool
    rcoef: float = 1e-4
    shots: list = field(default_factory=list)

    @property
    def ndim(self):
        return self.vp.ndim


def ricker(t, t0, f0):
    a = (np.pi * f0 * (t - t0)) ** 2
    return (1 - 2 * a) * np.exp(-a)


def smooth_model(shape, vmin, vmax, seed, blobs=4):
    """Seeded smooth velocity: linear trend in depth plus Gaussian blobs."""
    rng = np.random.default_rng(seed)
    grids = np.meshgrid(*[np.arange(n, dtype=np.float64) for n in shape], indexing="ij")
    depth = grids[-1] / max(shape[-1] - 1, 1)
    v = vmin + 0.6 * (vmax - vmin) * depth
    for _ in range(blobs):
        c = [rng.uniform(0, n - 1) for n in shape]
        s = rng.uniform(0.08, 0.2) * min(shape)
        amp = rng.uniform(-0.2, 0.2) * (vmax - vmin)
        r2 = sum((g - cc) ** 2 for g, cc in zip(grids, c))
        v = v + amp * np.exp(-0.5 * r2 / s ** 2)
    return np.asfortranarray(np.clip(v, vmin, vmax))


def stable_dt(vp, h, frac=0.6):
    return frac / (float(np.max(vp)) * np.sqrt(sum(1.0 / hh ** 2 for hh in h)))


def make_shot(case_h, extent, nt, dt, f0, src_pos, rec_pos, nsrc_tf=None):
    t = np.arange(nt) * dt
    src_pos = np.atleast_2d(np.asarray(src_pos, dtype=np.float64))
    tf = np.stack([ricker(t, 1.2 / f0 + 0.002 * k, f0) for k in range(src_pos.shape[0])], axis=1)
    return Shot(src_pos=src_pos, rec_pos=np.atleast_2d(np.asarray(rec_pos, dtype=np.float64)),
                tf=np.asfortranarray(tf), f0=f0, nt=nt)


def prepared(sw, case: Case, shot: Shot):
    """Indices, scaled float32 tf and float32 cpml block of one shot (the backend's inputs)."""
    si = sw.nearest_grid_points(shot.src_pos, case.h)
    ri = sw.nearest_grid_points(shot.rec_pos, case.h)
    scal = sw.scale_srctf(shot.tf, si, case.vp, case.h, case.dt)
    vmax = float(np.max(case.vp))
    parts = []
    for d in range(case.ndim):
        parts += sw._lib.cpml_coefficients(vmax, case.dt, case.halo, case.rcoef, case.h[d], shot.f0,
                                           case.freetop and d == case.ndim - 1)
    cp = np.concatenate(parts).astype(np.float32)
    return si, ri, scal, cp


# ---------------------------------------------------------------- oracle side
def oracle_cpml(oracle, case: Case, f0):
    return oracle.cpml_blocks(case.vp, case.h, case.dt, case.halo, case.rcoef, f0, case.freetop)


def oracle_forward(oracle, sw, case: Case, shot: Shot, f32=False):
    si, ri, scal, _ = prepared(sw, case, shot)
    return oracle.acoustic_forward(case.vp, case.h, case.dt, case.halo, oracle_cpml(oracle, case, shot.f0),
                                   scal.astype(np.float64), si, ri, f32=f32)


def oracle_gradient(oracle, sw, case: Case, shot: Shot, check_freq=1, mute_src=0, mute_rec=0, f32=False):
    si, ri, scal, _ = prepared(sw, case, shot)
    return oracle.acoustic_gradient(case.vp, case.h, case.dt, case.halo, oracle_cpml(oracle, case, shot.f0),
                                    scal.astype(np.float64), si, ri, shot.observed, invcov=shot.invcov,
                                    windows=shot.windows, check_freq=check_freq, mute_src=mute_src,
                                    mute_rec=mute_rec, src_pos=shot.src_pos, rec_pos=shot.rec_pos, f32=f32)


# ---------------------------------------------------------------- GPU side (C ABI)
class GpuRun:
    """Drives libswgb300 directly through its C ABI for one case."""

    def __init__(self, sw, case: Case, gradient=False, check_freq=1, mute_src=0, mute_rec=0, variant=0, tz=0,
                 bf16=False, precision=0):
        L = sw._lib
        self.sw, self.case, self.L = sw, case, L
        self.ctx = L.Context(0)
        prm = L.SwAcousticParams()
        prm.ndim = case.ndim
        for d in range(case.ndim):
            prm.n[d] = case.vp.shape[d]
            prm.h[d] = case.h[d]
        prm.dt, prm.halo, prm.rcoef, prm.freetop = case.dt, case.halo, case.rcoef, int(case.freetop)
        gp = L.SwGradParams()
        gp.check_freq, gp.mute_radius_src, gp.mute_radius_rec = check_freq, mute_src, mute_rec
        gp.snapshot_bf16 = int(bf16)  # 0 FP32, 1 BF16 recompute buffer, 2 also BF16 checkpoints
        self.h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.sw_wavesim_create(self.ctx.h, ctypes.byref(prm), int(gradient),
                                                      ctypes.byref(gp), ctypes.byref(self.h)), "create")
        self.precision = precision
        if precision:  # 1: compensated (double-FP32) forward steps, fact from the FP64 model
            self.ctx.check(self.ctx.lib.sw_wavesim_set_precision(self.h, int(precision)), "set_precision")
            vp64 = np.asfortranarray(case.vp, dtype=np.float64)
            self.ctx.check(self.ctx.lib.sw_wavesim_set_vp64(self.h, vp64.ctypes.data, 0), "set_vp64")
        else:
            vp32 = np.asfortranarray(case.vp, dtype=np.float32)
            self.ctx.check(self.ctx.lib.sw_wavesim_set_vp(self.h, vp32.ctypes.data, 0), "set_vp")
        if variant or tz:
            self.ctx.check(self.ctx.lib.sw_wavesim_set_tuning(self.h, int(tz), int(variant)), "set_tuning")

    def _structs(self, shots, grad):
        L = self.L
        arr = (L.SwAcousticShot * len(shots))()
        keep, outs = [], []
        for k, shot in enumerate(shots):
            si, ri, scal, cp = prepared(self.sw, self.case, shot)
            scal = np.asfortranarray(scal[: shot.nt])
            tr = np.zeros((shot.nt, ri.shape[0]), np.float32, order="F")
            st = arr[k]
            st.nt, st.nsrc, st.nrec = shot.nt, si.shape[0], ri.shape[0]
            st.src_idx, st.rec_idx, st.srctf, st.traces, st.cpml = (si.ctypes.data, ri.ctypes.data,
                                                                   scal.ctypes.data, tr.ctypes.data, cp.ctypes.data)
            items = [si, ri, scal, tr, cp]
            if self.precision:  # the FP64 coefficients of the compensated forward
                vmax = float(np.max(self.case.vp))
                parts = []
                for d in range(self.case.ndim):
                    parts += L.cpml_coefficients64(vmax, self.case.dt, self.case.halo, self.case.rcoef, self.case.h[d],
                                                   shot.f0, self.case.freetop and d == self.case.ndim - 1)
                cp64 = np.concatenate(parts)
                st.cpml64 = cp64.ctypes.data
                items.append(cp64)
            if grad:
                obs = np.asfortranarray(shot.observed, dtype=np.float32)
                st.observed = obs.ctypes.data
                items.append(obs)
                if shot.invcov is not None and np.ndim(shot.invcov) == 2:  # dense (nt, nt)
                    ic = np.asfortranarray(shot.invcov, dtype=np.float32)
                    st.invcov = ic.ctypes.data
                    items.append(ic)  # keeps the buffer alive until the call returns
                elif shot.invcov is not None:
                    ic = np.ascontiguousarray(shot.invcov, dtype=np.float32)
                    st.invcov_diag = ic.ctypes.data
                    items.append(ic)
                if shot.windows:
                    w = np.ascontiguousarray(np.array(shot.windows, dtype=np.int32).reshape(-1))
                    st.nwin, st.windows = len(shot.windows), w.ctypes.data
                    items.append(w)
                sp = np.asfortranarray(shot.src_pos)
                rp = np.asfortranarray(shot.rec_pos)
                st.src_pos, st.rec_pos = sp.ctypes.data, rp.ctypes.data
                items += [sp, rp]
            keep.append(items)
            outs.append(tr)
        return arr, keep, outs

    def forward(self, shots):
        arr, keep, outs = self._structs(shots, False)
        self.ctx.check(self.ctx.lib.sw_acoustic_forward(self.h, len(shots), arr, 0), "forward")
        return outs

    def gradient(self, shots):
        arr, keep, outs = self._structs(shots, True)
        g = np.zeros(self.case.vp.shape, np.float64, order="F")
        m = np.zeros(1, np.float64)
        self.ctx.check(self.ctx.lib.sw_acoustic_gradient(self.h, len(shots), arr, 0, g.ctypes.data,
                                                          m.ctypes.data), "gradient")
        return g, float(m[0]), outs

    def close(self):
        self.ctx.lib.sw_wavesim_destroy(self.h)
        self.ctx.close()


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
