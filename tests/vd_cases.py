"""Variable-density acoustic 2D test cases: seeded models and shots, and the
drivers that run one case through the oracle (FP64) and through libswgb300
(C ABI, sw_acoustic_vd_*)."""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

import __graft_entry__

sw = __graft_entry__.load_package()


def ricker(t, t0, f0):
    a = (math.pi * f0 * (t - t0)) ** 2
    return (1 - 2 * a) * np.exp(-a)


def gaussderiv(t, t0, f0):
    """gaussderivstf (src/utils/utils.jl:13)."""
    return (t - t0) * np.exp(-(math.pi * f0 * (t - t0)) ** 2)


@dataclass
class VDShot:
    src: np.ndarray            # (nsrc, 2) metres
    rec: np.ndarray            # (nrec, 2) metres
    tf: np.ndarray             # (nt, nsrc) unscaled
    f0: float

    @property
    def nt(self):
        return self.tf.shape[0]


@dataclass
class VDCase:
    vp: np.ndarray             # (nx, nz) Fortran order
    rho: np.ndarray
    h: float
    dt: float
    halo: int
    freetop: bool = False
    interp: int = 0            # 1/rho at the half points: 0 arithmetic, 1 harmonic
    rcoef: float = 1e-4
    shots: list = field(default_factory=list)

    @property
    def n(self):
        return self.vp.shape


def nearest(pos, h):
    return np.floor(np.atleast_2d(pos) / h + 1 + 0.5).astype(np.int32)


def scaled_tf(case: VDCase, shot: VDShot):
    """possrcrec_scaletf of the VD simulation (acou_forward.jl:66-80)."""
    si = nearest(shot.src, case.h)
    s = shot.tf / (case.h * case.h) * case.dt
    for k in range(s.shape[1]):
        i, j = si[k] - 1
        s[:, k] = s[:, k] * case.vp[i, j] ** 2 * case.rho[i, j]
    return np.asfortranarray(s)


def cpml(case: VDCase, shot: VDShot):
    import oracle
    return oracle.cpml_blocks(case.vp, (case.h, case.h), case.dt, case.halo, case.rcoef, shot.f0, case.freetop)


def oracle_forward(case, shot, f32=False, snapevery=0):
    import oracle
    return oracle.vd_forward(case.vp, case.rho, (case.h, case.h), case.dt, case.halo, cpml(case, shot),
                             scaled_tf(case, shot), nearest(shot.src, case.h), nearest(shot.rec, case.h),
                             interp=case.interp, f32=f32, snapevery=snapevery)


def oracle_gradient(case, shot, observed, *, check_freq=1, invcov=None, windows=(), mute_src=0, mute_rec=0,
                    f32=False, ccts_dt=None):
    import oracle
    return oracle.vd_gradient(case.vp, case.rho, (case.h, case.h), case.dt, case.halo, cpml(case, shot),
                              scaled_tf(case, shot), nearest(shot.src, case.h), nearest(shot.rec, case.h),
                              observed, interp=case.interp, invcov=invcov, windows=windows, check_freq=check_freq,
                              mute_src=mute_src, mute_rec=mute_rec, src_pos=shot.src, rec_pos=shot.rec, f32=f32,
                              ccts_dt=ccts_dt)


class GpuVD:
    """One sw_acoustic_vd through the C ABI (host buffers)."""

    def __init__(self, lib_ctx, case: VDCase, gradient=False, check_freq=1, mute_src=0, mute_rec=0, precision=0):
        self.ctx = lib_ctx
        self.case = case
        L = sw._lib
        prm = L.SwAcousticParams()
        prm.ndim = 2
        prm.n[0], prm.n[1], prm.n[2] = case.vp.shape[0], case.vp.shape[1], 1
        prm.h[0], prm.h[1], prm.h[2] = case.h, case.h, 1.0
        prm.dt, prm.halo, prm.rcoef, prm.freetop = case.dt, case.halo, case.rcoef, int(case.freetop)
        gp = L.SwGradParams()
        gp.check_freq, gp.mute_radius_src, gp.mute_radius_rec, gp.compute_misfit = check_freq, mute_src, mute_rec, 1
        self.h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.sw_acoustic_vd_create(self.ctx.h, ctypes.byref(prm), int(case.interp),
                                                          int(gradient), ctypes.byref(gp), ctypes.byref(self.h)),
                       "sw_acoustic_vd_create")
        self.precision = precision
        if precision:  # compensated forward: the factors from the FP64 model
            self.ctx.check(self.ctx.lib.sw_acoustic_vd_set_precision(self.h, int(precision)), "set_precision")
            vp64 = np.asfortranarray(case.vp, dtype=np.float64)
            rho64 = np.asfortranarray(case.rho, dtype=np.float64)
            self.ctx.check(self.ctx.lib.sw_acoustic_vd_set_material64(self.h, vp64.ctypes.data, rho64.ctypes.data),
                           "sw_acoustic_vd_set_material64")
        else:
            vp = np.asfortranarray(case.vp, dtype=np.float32)
            rho = np.asfortranarray(case.rho, dtype=np.float32)
            self.ctx.check(self.ctx.lib.sw_acoustic_vd_set_material(self.h, vp.ctypes.data, rho.ctypes.data),
                           "sw_acoustic_vd_set_material")

    def close(self):
        if self.h:
            self.ctx.lib.sw_acoustic_vd_destroy(self.h)
            self.h = ctypes.c_void_p()

    def _structs(self, shots, observed=None, invcov=None, windows=None, ccts_dt=None):
        L = sw._lib
        keep, structs = [], (L.SwAcousticShot * len(shots))()
        for k, shot in enumerate(shots):
            si = np.asfortranarray(nearest(shot.src, self.case.h))
            ri = np.asfortranarray(nearest(shot.rec, self.case.h))
            tf = np.asfortranarray(scaled_tf(self.case, shot), dtype=np.float32)
            nrec = shot.rec.shape[0]
            tr = np.zeros((shot.nt, nrec), dtype=np.float32, order="F")
            cp = cpml(self.case, shot).astype(np.float32)
            st = structs[k]
            st.nt, st.nsrc, st.nrec = shot.nt, shot.src.shape[0], nrec
            st.src_idx, st.srctf, st.rec_idx = si.ctypes.data, tf.ctypes.data, ri.ctypes.data
            st.traces, st.cpml = tr.ctypes.data, cp.ctypes.data
            arrs = [si, ri, tf, tr, cp]
            if self.precision:  # FP64 coefficients of the compensated forward
                cp64 = np.ascontiguousarray(cpml(self.case, shot), dtype=np.float64)
                st.cpml64 = cp64.ctypes.data
                arrs.append(cp64)
            if observed is not None:
                obs = np.asfortranarray(observed[k], dtype=np.float32)
                st.observed = obs.ctypes.data
                arrs.append(obs)
                if invcov is not None and invcov[k] is not None:
                    if np.ndim(invcov[k]) == 2:
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
                if ccts_dt is not None:
                    st.misfit_kind, st.misfit_dt = 1, float(ccts_dt)
            keep.append((tr, arrs))
        return structs, keep

    def forward(self, shots):
        structs, keep = self._structs(shots)
        self.ctx.check(self.ctx.lib.sw_acoustic_vd_forward(self.h, len(shots), structs, 0), "sw_acoustic_vd_forward")
        return [k[0].astype(np.float64) for k in keep]

    def forward_snapshots(self, shots, snapevery):
        structs, keep = self._structs(shots)
        nx, nz = self.case.vp.shape
        B = nx * nz + (nx - 1) * nz + nx * (nz - 1)
        bufs = [np.zeros((s.nt // snapevery) * B, dtype=np.float32) for s in shots]
        ptrs = (ctypes.c_void_p * len(shots))(*[b.ctypes.data for b in bufs])
        self.ctx.check(self.ctx.lib.sw_acoustic_vd_forward_snapshots(self.h, len(shots), structs, 0, snapevery, ptrs),
                       "sw_acoustic_vd_forward_snapshots")
        out = []
        for b in bufs:
            snaps = []
            for q in range(len(b) // B):
                blk = b[q * B:(q + 1) * B].astype(np.float64)
                snaps.append((blk[:nx * nz].reshape((nx, nz), order="F"),
                              blk[nx * nz:nx * nz + (nx - 1) * nz].reshape((nx - 1, nz), order="F"),
                              blk[nx * nz + (nx - 1) * nz:].reshape((nx, nz - 1), order="F")))
            out.append(snaps)
        return [k[0].astype(np.float64) for k in keep], out

    def gradient(self, shots, observed, invcov=None, windows=None, ccts_dt=None):
        structs, keep = self._structs(shots, observed, invcov, windows, ccts_dt)
        nx, nz = self.case.vp.shape
        g = {k: np.zeros((nx, nz), dtype=np.float64, order="F") for k in ("vp", "rho")}
        m = np.zeros(1)
        self.ctx.check(self.ctx.lib.sw_acoustic_vd_gradient(self.h, len(shots), structs, 0, g["vp"].ctypes.data,
                                                            g["rho"].ctypes.data, m.ctypes.data),
                       "sw_acoustic_vd_gradient")
        return g, float(m[0]), [k[0].astype(np.float64) for k in keep]


def smooth_vd(nx, nz, h, seed=0):
    """vp 1800-3200 m/s and rho 1700-2500 kg/m^3 from seeded smooth fields
    (rho loosely follows vp, as Gardner's relation would)."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx)[:, None] * h
    z = np.arange(nz)[None, :] * h
    vp = 1800.0 + 1200.0 * z / z.max() + 0.0 * x
    for _ in range(3):
        cx, cz = rng.uniform(0, x.max()), rng.uniform(0, z.max())
        s = rng.uniform(4, 10) * h
        vp = vp + rng.uniform(-200, 200) * np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (2 * s * s))
    rho = 1700.0 + 600.0 * (vp - vp.min()) / (vp.max() - vp.min())
    rho = rho + 100.0 * np.sin(x / (9 * h)) * np.cos(z / (6 * h))
    return np.asfortranarray(vp), np.asfortranarray(rho)


def stable_dt(vp, h, frac=0.5):
    """CFL with the 7/6 factor of the 4th-order stencil (acou_models.jl:240-251)."""
    return frac / (float(np.max(vp)) * math.sqrt(2.0 / h ** 2) * 7 / 6)


def small_case(nt=400, seed=0, interp=0, freetop=False, nx=120, nz=100, halo=20, nsrc=1, f0=15.0):
    h = 5.0
    vp, rho = smooth_vd(nx, nz, h, seed)
    dt = stable_dt(vp, h)
    ez = (nz - 1) * h
    sz = 12 * h if freetop else 0.5 * ez
    src = np.array([[nx * h * 0.45 + 1.3 + 17.0 * k, sz + 0.7] for k in range(nsrc)])
    rz = 8 * h if freetop else 0.3 * ez
    rec = np.array([[x, rz] for x in np.linspace(0.2 * nx * h, 0.8 * nx * h, 9)])
    t = np.arange(nt) * dt
    tf = np.stack([ricker(t, 1.2 / f0 + 0.003 * k, f0) for k in range(nsrc)], axis=1)
    shot = VDShot(src, rec, tf, f0)
    return VDCase(vp, rho, h, dt, halo, freetop=freetop, interp=interp, shots=[shot])


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
