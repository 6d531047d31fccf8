"""Elastic 2D test cases: seeded models, shots and the drivers that run one
case through the oracle (FP64) and through libswgb300 (C ABI)."""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

import __graft_entry__

sw = __graft_entry__.load_package()
E = __import__(sw.__name__ + ".elastic", fromlist=["elastic"])


def ricker(nt, dt, f0, t0=None):
    t = np.arange(nt) * dt
    t0 = 2.0 / f0 if t0 is None else t0
    a = (math.pi * f0 * (t - t0)) ** 2
    return (1 - 2 * a) * np.exp(-a)


@dataclass
class ElShot:
    kind: str                  # "mt" or "force"
    src: np.ndarray            # (nsrc, 2) metres
    rec: np.ndarray            # (nrec, 2) metres
    nt: int
    f0: float = 15.0
    momtens: list = field(default_factory=lambda: [(1.0, 1.0, 0.0)])
    amp: float = 1.0


@dataclass
class ElCase:
    nx: int
    nz: int
    h: float
    dt: float
    halo: int
    lam: np.ndarray
    mu: np.ndarray
    rho: np.ndarray
    shots: list
    freetop: bool = False
    sinc: bool = True
    interp_rho: int = 0
    interp_mu: int = 0
    rcoef: float = 1e-4


def homogeneous(nx, nz, vp=3000.0, rho=2200.0):
    vs = vp / math.sqrt(3.0)
    lam = np.full((nx, nz), rho * (vp ** 2 - 2 * vs ** 2))
    mu = np.full((nx, nz), rho * vs ** 2)
    return lam, mu, np.full((nx, nz), rho)


def smooth(nx, nz, h, seed=0):
    """vp 2000-3200, vs = vp/sqrt(3)*U(0.9,1.0), rho 1800-2500 from seeded smooth fields."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx)[:, None] * h
    z = np.arange(nz)[None, :] * h
    vp = 2000.0 + 1200.0 * z / z.max()
    for _ in range(3):
        cx, cz = rng.uniform(0, x.max()), rng.uniform(0, z.max())
        s = rng.uniform(4, 10) * h
        vp = vp + rng.uniform(-200, 200) * np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (2 * s * s))
    vs = vp / math.sqrt(3.0) * (0.9 + 0.1 * (0.5 + 0.5 * np.sin(x / (7 * h)) * np.cos(z / (5 * h))))
    rho = 1800.0 + 700.0 * (vp - vp.min()) / (vp.max() - vp.min())
    lam = rho * (vp ** 2 - 2 * vs ** 2)
    mu = rho * vs ** 2
    return lam, mu, rho


def stable_dt(lam, mu, rho, h, frac=0.5):
    vmax = float(np.max(np.sqrt((lam + 2 * mu) / rho)))
    return frac / (vmax * math.sqrt(2.0 / h ** 2) * 7 / 6)


def tables(case: ElCase, shot: ElShot):
    n, hh = (case.nx, case.nz), (case.h, case.h)
    h = case.h
    if case.sinc:
        sp = lambda pos, sh, mir: E.spread_positions(n, hh, pos, shift=sh, mirror=mir)  # noqa: E731
        if shot.kind == "mt":
            src = [sp(shot.src, (0.0, 0.0), True), sp(shot.src, (h / 2, h / 2), True)]
        else:
            src = [sp(shot.src, (h / 2, 0.0), False), sp(shot.src, (0.0, h / 2), False)]
        rec = [sp(shot.rec, (h / 2, 0.0), False), sp(shot.rec, (0.0, h / 2), False)]
    else:
        ps = sw.nearest_grid_points(shot.src, hh)
        pr = sw.nearest_grid_points(shot.rec, hh)
        one = lambda idx: [(np.array([row], np.int32), np.ones(1)) for row in idx]  # noqa: E731
        src, rec = [one(ps), one(ps)], [one(pr), one(pr)]
    return src, rec


def srctf(case: ElCase, shot: ElShot):
    w = ricker(shot.nt, case.dt, shot.f0) * shot.amp / (case.h * case.h)
    ns = shot.src.shape[0]
    if shot.kind == "mt":
        return np.repeat(w[:, None], ns, axis=1)
    tf = np.zeros((shot.nt, 2, ns))
    tf[:, 0, :] = w[:, None]
    tf[:, 1, :] = 0.5 * w[:, None]
    return tf


def cpml(case: ElCase, shot: ElShot):
    import oracle
    vp = np.sqrt((case.lam + 2 * case.mu) / case.rho)
    return oracle.cpml_blocks(vp, (case.h, case.h), case.dt, case.halo, case.rcoef, shot.f0, case.freetop)


def oracle_shot(case, shot):
    src, rec = tables(case, shot)
    d = dict(kind=shot.kind, srctf=srctf(case, shot), src_tables=src, rec_tables=rec)
    if shot.kind == "mt":
        d["momtens"] = np.array(shot.momtens, dtype=np.float64).reshape(-1, 3)
    return d


def oracle_forward(case, shot, f32=False):
    import oracle
    return oracle.elastic_forward(case.lam, case.mu, case.rho, (case.h, case.h), case.dt, case.halo, case.freetop,
                                  cpml(case, shot), oracle_shot(case, shot), interp_rho=case.interp_rho,
                                  interp_mu=case.interp_mu, f32=f32)


def oracle_gradient(case, shot, observed, *, check_freq=1, invcov=None, windows=(), mute_src=0, mute_rec=0,
                    f32=False, ccts_dt=None):
    import oracle
    return oracle.elastic_gradient(case.lam, case.mu, case.rho, (case.h, case.h), case.dt, case.halo, case.freetop,
                                   cpml(case, shot), oracle_shot(case, shot), observed, invcov=invcov,
                                   windows=windows, check_freq=check_freq, mute_src=mute_src, mute_rec=mute_rec,
                                   src_pos=shot.src, rec_pos=shot.rec, interp_rho=case.interp_rho,
                                   interp_mu=case.interp_mu, f32=f32, ccts_dt=ccts_dt)


class GpuElastic:
    """One sw_elastic through the C ABI (host buffers)."""

    def __init__(self, lib_ctx, case: ElCase, gradient=False, check_freq=1, mute_src=0, mute_rec=0):
        self.ctx = lib_ctx
        self.case = case
        L = sw._lib
        prm = L.SwElasticParams()
        prm.n[0], prm.n[1] = case.nx, case.nz
        prm.h[0], prm.h[1] = case.h, case.h
        prm.dt, prm.halo, prm.rcoef, prm.freetop = case.dt, case.halo, case.rcoef, int(case.freetop)
        prm.interp_rho, prm.interp_mu = case.interp_rho, case.interp_mu
        gp = L.SwGradParams()
        gp.check_freq, gp.mute_radius_src, gp.mute_radius_rec = check_freq, mute_src, mute_rec
        self.h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.sw_elastic_create(self.ctx.h, ctypes.byref(prm), int(gradient), ctypes.byref(gp),
                                                      ctypes.byref(self.h)), "sw_elastic_create")
        arrs = [np.asfortranarray(a, dtype=np.float32) for a in (case.lam, case.mu, case.rho)]
        self.ctx.check(self.ctx.lib.sw_elastic_set_material(self.h, *(a.ctypes.data for a in arrs)),
                       "sw_elastic_set_material")

    def close(self):
        if self.h:
            self.ctx.lib.sw_elastic_destroy(self.h)
            self.h = ctypes.c_void_p()

    def _structs(self, shots, observed=None, invcov=None, windows=None, ccts_dt=None):
        L = sw._lib
        keep, structs = [], (L.SwElasticShot * len(shots))()
        for k, shot in enumerate(shots):
            src, rec = tables(self.case, shot)
            tf = np.asfortranarray(srctf(self.case, shot), dtype=np.float32)
            nrec = shot.rec.shape[0]
            tr = np.zeros((shot.nt, 2, nrec), dtype=np.float32, order="F")
            cp = cpml(self.case, shot).astype(np.float32)
            st = structs[k]
            st.nt, st.kind, st.nsrc, st.nrec = shot.nt, 0 if shot.kind == "mt" else 1, shot.src.shape[0], nrec
            st.srctf, st.traces, st.cpml = tf.ctypes.data, tr.ctypes.data, cp.ctypes.data
            arrs = [tf, tr, cp]
            if shot.kind == "mt":
                m3 = np.ascontiguousarray(np.array(shot.momtens, dtype=np.float32).reshape(-1, 3))
                st.momtens = m3.ctypes.data
                arrs.append(m3)
            for t in range(2):
                for tab, tgt in ((src[t], st.src[t]), (rec[t], st.rec[t])):
                    off, ij, coef = E._table(tab)
                    tgt.offsets, tgt.ij, tgt.coef = off.ctypes.data, ij.ctypes.data, coef.ctypes.data
                    arrs += [off, ij, coef]
            if observed is not None:
                obs = np.asfortranarray(observed[k], dtype=np.float32)
                st.observed = obs.ctypes.data
                arrs.append(obs)
                if ccts_dt is not None:
                    st.misfit_kind, st.misfit_dt = 1, ccts_dt
                if invcov is not None and invcov[k] is not None:
                    if np.ndim(invcov[k]) == 2:  # dense (nt, nt)
                        ic = np.asfortranarray(invcov[k], dtype=np.float32)
                        st.invcov = ic.ctypes.data
                    else:
                        ic = np.ascontiguousarray(invcov[k], dtype=np.float32)
                        st.invcov_diag = ic.ctypes.data
                    arrs.append(ic)
                if windows is not None and windows[k]:
                    w = np.ascontiguousarray(np.array(windows[k], dtype=np.int32).reshape(-1))
                    st.nwin, st.windows = len(windows[k]), w.ctypes.data
                    arrs.append(w)
                spp = np.asfortranarray(shot.src, dtype=np.float64)
                rpp = np.asfortranarray(shot.rec, dtype=np.float64)
                st.src_pos, st.rec_pos = spp.ctypes.data, rpp.ctypes.data
                arrs += [spp, rpp]
            keep.append((tr, arrs))
        return structs, keep

    def forward(self, shots):
        structs, keep = self._structs(shots)
        self.ctx.check(self.ctx.lib.sw_elastic_forward(self.h, len(shots), structs, 0), "sw_elastic_forward")
        return [k[0].astype(np.float64) for k in keep]

    def gradient(self, shots, observed, invcov=None, windows=None, ccts_dt=None):
        structs, keep = self._structs(shots, observed, invcov, windows, ccts_dt)
        nx, nz = self.case.nx, self.case.nz
        g = {k: np.zeros((nx, nz), dtype=np.float64, order="F") for k in ("rho", "lambda", "mu")}
        m = np.zeros(1)
        self.ctx.check(self.ctx.lib.sw_elastic_gradient(self.h, len(shots), structs, 0, g["rho"].ctypes.data,
                                                         g["lambda"].ctypes.data, g["mu"].ctypes.data, m.ctypes.data),
                       "sw_elastic_gradient")
        return g, float(m[0]), [k[0].astype(np.float64) for k in keep]


def small_case(kind="mt", freetop=False, sinc=True, nt=400, seed=0, interp=(0, 0), nx=120, nz=100, halo=20):
    h = 5.0
    lam, mu, rho = smooth(nx, nz, h, seed)
    dt = stable_dt(lam, mu, rho, h)
    ez = (nz - 1) * h
    sz = 12 * h if freetop else 0.5 * ez
    src = np.array([[nx * h * 0.45 + 1.3, sz + 0.7]])
    rz = 8 * h if freetop else 0.3 * ez
    rec = np.array([[x, rz] for x in np.linspace(0.2 * nx * h, 0.8 * nx * h, 9)])
    shot = ElShot(kind, src, rec, nt)
    return ElCase(nx, nz, h, dt, halo, lam, mu, rho, [shot], freetop=freetop, sinc=sinc, interp_rho=interp[0],
                  interp_mu=interp[1])


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
