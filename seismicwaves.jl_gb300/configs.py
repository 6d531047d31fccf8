"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference publishes no benchmark data set; these generators produce
models, acquisition geometries and source wavelets of the stated sizes and
value ranges (numpy PCG64, fixed seeds).  Each returns a ``Workload`` whose
shots are given as positions in metres and unscaled source time functions,
exactly what a SeismicWaves.jl user passes to ScalarSources/ScalarReceivers.

  acoustic2d_201       201 x 201, h = 5 m, Gaussian +300 m/s anomaly, 1 shot, 101 receivers, nt = 1000
  acoustic2d_801       801 x 801, h = 5 m, gradient + 8 blobs, 1 shot, 401 receivers, nt = 3000, K = 50
  acoustic2d_2001x801  2001 x 801, h = 10 m, 12 layers, 64 shots, 50-300 receivers, nt in [2000, 4000], K = 50
  acoustic3d_400       400^3, h = 10 m, smooth random 1800-4000 m/s, 16 shots, 40 x 40 receivers, nt = 2000, K = 100
  acoustic_vd2d_2001x801  the acoustic2d_2001x801 model and shots with a density from Gardner's relation
                       rho = 310 vp^0.25 (kg/m^3) and the variable-density scheme's CFL (7/6 factor)
  elastic2d_1200x600   1200 x 600, h = 5 m, vp 2000-4500, vs = vp/sqrt(3) * U(0.9, 1.0), rho 1800-2700 (smooth
                       seeded fields), 32 explosive moment-tensor shots, 300 receivers, nt = 4000, 15 Hz, K = 50
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class WShot:
    src_pos: np.ndarray   # (1, ndim) metres
    rec_pos: np.ndarray   # (nrec, ndim) metres
    nt: int
    f0: float
    t0: float

    def stf(self, dt):
        t = np.arange(self.nt) * dt
        a = (np.pi * self.f0 * (t - self.t0)) ** 2
        return ((1 - 2 * a) * np.exp(-a)).reshape(self.nt, 1)


@dataclass
class Workload:
    name: str
    vp: np.ndarray        # Fortran order
    h: tuple
    dt: float
    halo: int
    freetop: bool
    check_freq: int
    shots: list = field(default_factory=list)
    vp_observed: np.ndarray | None = None  # model that generates the observed data
    rho: np.ndarray | None = None          # variable-density workloads
    rho_observed: np.ndarray | None = None

    @property
    def gridpoints(self):
        return int(np.prod(self.vp.shape))

    def point_steps(self):
        return sum(self.gridpoints * s.nt for s in self.shots)


def _dt(vp, h, frac=0.6):
    return frac / (float(np.max(vp)) * np.sqrt(sum(1.0 / hh ** 2 for hh in h)))


def _box_smooth(a, w):
    """Separable moving average over w cells (edges replicated)."""
    out = a
    for ax in range(a.ndim):
        pad = [(0, 0)] * a.ndim
        pad[ax] = (w // 2, w - 1 - w // 2)
        p = np.pad(out, pad, mode="edge")
        c = np.cumsum(p, axis=ax, dtype=np.float64)
        c = np.concatenate([np.zeros_like(np.take(c, [0], axis=ax)), c], axis=ax)
        n = out.shape[ax]
        out = (np.take(c, range(w, w + n), axis=ax) - np.take(c, range(0, n), axis=ax)) / w
    return out


def _gauss_smooth(a, sigma):
    """Separable Gaussian filter (truncated at 4 sigma, edges replicated)."""
    try:  # same filter, much faster on large grids
        from scipy.ndimage import gaussian_filter
        return gaussian_filter(a, sigma, mode="nearest", truncate=4.0)
    except ImportError:
        pass
    r = int(4 * sigma + 0.5)
    x = np.arange(-r, r + 1)
    k = np.exp(-0.5 * (x / sigma) ** 2)
    k /= k.sum()
    out = a
    for ax in range(a.ndim):
        pad = [(0, 0)] * a.ndim
        pad[ax] = (r, r)
        p = np.pad(out, pad, mode="edge")
        acc = np.zeros_like(out)
        for i, w in enumerate(k):
            acc += w * np.take(p, range(i, i + out.shape[ax]), axis=ax)
        out = acc
    return out


def acoustic2d_201() -> Workload:
    nx = nz = 201
    h = 5.0
    x = np.arange(nx) * h
    z = np.arange(nz) * h
    X, Z = np.meshgrid(x, z, indexing="ij")
    r2 = (X - x[-1] / 2) ** 2 + (Z - z[-1] / 2) ** 2
    vp = np.asfortranarray(2000.0 + 300.0 * np.exp(-r2 / (2 * 100.0 ** 2)))
    rec = np.stack([np.arange(0, 1001, 10.0), np.full(101, 20.0)], 1)
    shot = WShot(np.array([[500.0, 25.0]]), rec, 1000, 12.0, 2 / 12.0)
    return Workload("acoustic2d_201", vp, (h, h), _dt(vp, (h, h)), 20, False, 1, [shot])


def acoustic2d_801(seed: int = 1) -> Workload:
    nx = nz = 801
    h = 5.0
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * h
    z = np.arange(nz) * h
    X, Z = np.meshgrid(x, z, indexing="ij")
    vp = 1500.0 + 2000.0 * Z / z[-1]
    for _ in range(8):
        cx, cz = rng.uniform(0, x[-1]), rng.uniform(0, z[-1])
        s = rng.uniform(50.0, 200.0)
        amp = rng.uniform(-300.0, 300.0)
        vp = vp + amp * np.exp(-((X - cx) ** 2 + (Z - cz) ** 2) / (2 * s ** 2))
    vp = np.asfortranarray(np.clip(vp, 1500.0, 3500.0))
    rec = np.stack([np.linspace(0.0, x[-1], 401), np.full(401, 20.0)], 1)
    shot = WShot(np.array([[2000.0, 20.0]]), rec, 3000, 10.0, 1.2 / 10.0)
    return Workload("acoustic2d_801", vp, (h, h), _dt(vp, (h, h)), 20, False, 50, [shot],
                    vp_observed=np.asfortranarray(vp * 1.05))


def _layered(nx, nz, h, seed):
    rng = np.random.default_rng(seed)
    nl = 12
    th = rng.uniform(0.5, 1.5, nl)
    bounds = np.concatenate([[0], np.cumsum(th) / th.sum() * nz]).astype(int)
    vlay = np.linspace(1500.0, 4500.0, nl)
    v = np.zeros((nx, nz))
    for k in range(nl):
        v[:, bounds[k]:bounds[k + 1]] = vlay[k]
    return v


def acoustic2d_2001x801(seed: int = 3, nshots: int = 64) -> Workload:
    nx, nz, h = 2001, 801, 10.0
    rng = np.random.default_rng(seed)
    v = _layered(nx, nz, h, seed)
    noise = _box_smooth(rng.standard_normal((nx, nz)), 5)
    vp = np.asfortranarray(np.clip(v * (1 + 0.03 * noise / max(noise.std(), 1e-12)), 1400.0, 4700.0))
    noise2 = _box_smooth(np.random.default_rng(seed + 1000).standard_normal((nx, nz)), 5)
    vobs = np.asfortranarray(np.clip(v * (1 + 0.03 * noise2 / max(noise2.std(), 1e-12)), 1400.0, 4700.0))
    ext = (nx - 1) * h
    shots = []
    xs = np.linspace(0.05 * ext, 0.95 * ext, nshots)
    for s in range(nshots):
        nrec = int(rng.integers(50, 301))
        nt = int(rng.integers(2000, 4001))
        rec = np.stack([np.linspace(0.02 * ext, 0.98 * ext, nrec), np.full(nrec, 20.0)], 1)
        shots.append(WShot(np.array([[xs[s], 20.0]]), rec, nt, 8.0, 1.2 / 8.0))
    dt = _dt(np.maximum(vp, vobs), (h, h))
    return Workload("acoustic2d_2001x801", vp, (h, h), dt, 20, False, 50, shots, vp_observed=vobs)


def acoustic_vd2d_2001x801(seed: int = 3, nshots: int = 64) -> Workload:
    w = acoustic2d_2001x801(seed, nshots)
    w.name = "acoustic_vd2d_2001x801"
    w.rho = np.asfortranarray(310.0 * w.vp ** 0.25)
    w.rho_observed = np.asfortranarray(310.0 * w.vp_observed ** 0.25)
    w.dt = _dt(np.maximum(w.vp, w.vp_observed), w.h) * 6 / 7
    return w


def acoustic3d_400(seed: int = 5, n: int = 400, nshots_side: int = 4, patch: int = 40, nt: int = 2000) -> Workload:
    h = 10.0
    rng = np.random.default_rng(seed)
    f = _gauss_smooth(rng.standard_normal((n, n, n)).astype(np.float64), 8.0)
    f = (f - f.min()) / max(f.max() - f.min(), 1e-12)
    vp = np.asfortranarray(1800.0 + 2200.0 * f)
    ext = (n - 1) * h
    shots = []
    cs = np.linspace(0.2 * ext, 0.8 * ext, nshots_side)
    for cx in cs:
        for cy in cs:
            off = (np.arange(patch) - (patch - 1) / 2) * 2 * h
            RX, RY = np.meshgrid(cx + off, cy + off, indexing="ij")
            rec = np.stack([RX.ravel(), RY.ravel(), np.full(patch * patch, 20.0)], 1)
            shots.append(WShot(np.array([[cx, cy, 20.0]]), rec, nt, 10.0, 1.2 / 10.0))
    return Workload("acoustic3d_400", vp, (h, h, h), _dt(vp, (h, h, h)), 20, False, 100, shots,
                    vp_observed=np.asfortranarray(vp * 1.03))


@dataclass
class ElasticWorkload:
    name: str
    lam: np.ndarray       # Fortran order (nx, nz)
    mu: np.ndarray
    rho: np.ndarray
    h: tuple
    dt: float
    halo: int
    freetop: bool
    check_freq: int
    shots: list = field(default_factory=list)
    observed_model: tuple | None = None  # (lam, mu, rho) that generates the observed data
    momtens: tuple = (1.0, 1.0, 0.0)     # Mxx, Mzz, Mxz (explosive)

    @property
    def gridpoints(self):
        return int(np.prod(self.lam.shape))

    def point_steps(self):
        return sum(self.gridpoints * s.nt for s in self.shots)

    @property
    def vp(self):
        return np.sqrt((self.lam + 2 * self.mu) / self.rho)


def _smooth_field(shape, sigma, seed):
    f = _gauss_smooth(np.random.default_rng(seed).standard_normal(shape), sigma)
    return (f - f.min()) / max(f.max() - f.min(), 1e-12)


def _elastic_model(nx, nz, seed):
    vp = 2000.0 + 2500.0 * _smooth_field((nx, nz), 20.0, seed)
    vs = vp / np.sqrt(3.0) * (0.9 + 0.1 * _smooth_field((nx, nz), 20.0, seed + 1))
    rho = 1800.0 + 900.0 * _smooth_field((nx, nz), 20.0, seed + 2)
    lam = rho * (vp ** 2 - 2 * vs ** 2)
    mu = rho * vs ** 2
    return tuple(np.asfortranarray(a) for a in (lam, mu, rho))


def elastic2d_1200x600(seed: int = 7, nshots: int = 32, nrec: int = 300, nt: int = 4000) -> ElasticWorkload:
    nx, nz, h = 1200, 600, 5.0
    lam, mu, rho = _elastic_model(nx, nz, seed)
    # observed model: the simulated one with 3 % smooth perturbations (a second seed)
    pert = 1.0 + 0.03 * (2.0 * _smooth_field((nx, nz), 20.0, seed + 200) - 1.0)
    obs = (np.asfortranarray(lam * pert), np.asfortranarray(mu * pert), rho)
    vmax = max(float(np.max(np.sqrt((lam + 2 * mu) / rho))), float(np.max(np.sqrt((obs[0] + 2 * obs[1]) / rho))))
    dt = 0.6 / (vmax * np.sqrt(2.0 / h ** 2) * 7.0 / 6.0)  # CFL number 0.6 with the 7/6 factor
    ext = (nx - 1) * h
    shots = []
    for x in np.linspace(0.1 * ext, 0.9 * ext, nshots):
        rec = np.stack([np.linspace(0.05 * ext, 0.95 * ext, nrec), np.full(nrec, 120.0)], 1)
        shots.append(WShot(np.array([[x, 150.0]]), rec, nt, 15.0, 1.2 / 15.0))
    return ElasticWorkload("elastic2d_1200x600", lam, mu, rho, (h, h), float(dt), 20, False, 50, shots,
                           observed_model=obs)


WORKLOADS = {
    "acoustic2d_201": acoustic2d_201,
    "acoustic2d_801": acoustic2d_801,
    "acoustic2d_2001x801": acoustic2d_2001x801,
    "acoustic_vd2d_2001x801": acoustic_vd2d_2001x801,
    "acoustic3d_400": acoustic3d_400,
    "elastic2d_1200x600": elastic2d_1200x600,
}
