"""Host-side mirror of SeismicWaves.jl's isotropic elastic 2D (P-SV) API over libswgb300.

Names, argument meanings and checks follow the reference (SeismicWaves.jl
v0.9.0):

    InputParametersElastic, ElasticIsoMaterialProperties, MomentTensor2D,
    MomentTensorSources, ExternalForceSources, VectorReceivers,
    MomentTensorShot, ExternalForceShot, ArithmeticAverageInterpolation,
    HarmonicAverageInterpolation, spread_positions, ElasticIsoCPMLWaveSimulation

Host logic kept from the reference: material checks and the CFL number with
the 7/6 factor (src/models/elastic/ela_models.jl:94-141), position checks
(src/utils/checks.jl:43-94), C-PML coefficients per shot (init_bdc!,
src/models/elastic/ela_init_bc.jl:7-40, computed by the library), the sinc
source/receiver spreading (spread_positions, src/utils/utils.jl:62-214) or the
nearest grid point (ela_models.jl:6-90), and the source scaling 1/(dx dz).
Time stepping, checkpointing, adjoint, correlation, back-interpolation,
muting and the sums over shots run on the GPU, all shots of a call batched.

Divergence from the reference, on purpose: as for the acoustic path,
CPMLBoundaryConditionParameters.vel_max is honoured (ela_init_bc.jl:13 reads
it as the acoustic code does); fields are FP32 whatever the input precision.
"""
from __future__ import annotations

import copy
import ctypes
import logging
import math
import warnings
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib

log = logging.getLogger("seismicwaves_gb300")


class InputParametersElastic:
    """src/models/elastic/ela_params.jl:1-34."""

    def __init__(self, ntimesteps: int, dt: float, gridsize: Sequence[int], gridspacing: Sequence[float], boundcond):
        assert len(gridsize) <= 3, "Dimensionality must be less than or equal to 3!"
        assert all(n > 0 for n in gridsize), "All numbers of grid points must be positive!"
        assert all(h > 0 for h in gridspacing), "All grid spacings must be positive!"
        assert ntimesteps > 0, "Number of timesteps must be positive!"
        assert dt > 0, "Timestep size must be positive!"
        self.ntimesteps, self.dt = int(ntimesteps), float(dt)
        self.gridsize = tuple(int(n) for n in gridsize)
        self.gridspacing = tuple(float(h) for h in gridspacing)
        self.boundcond = boundcond


class ArithmeticAverageInterpolation:
    """src/utils/interpolations.jl:31 (code 0 for the library)."""
    code = 0


class HarmonicAverageInterpolation:
    """src/utils/interpolations.jl:33 (code 1 for the library)."""
    code = 1


@dataclass
class ElasticIsoMaterialProperties:
    """src/models/elastic/ela_material_properties.jl:9-22."""
    λ: np.ndarray
    μ: np.ndarray
    ρ: np.ndarray
    interp_method_ρ: object = None
    interp_method_λ: object = None
    interp_method_μ: object = None

    def __post_init__(self):
        if self.interp_method_ρ is None:
            self.interp_method_ρ = ArithmeticAverageInterpolation()
        if self.interp_method_λ is None:
            self.interp_method_λ = HarmonicAverageInterpolation()
        if self.interp_method_μ is None:
            self.interp_method_μ = ArithmeticAverageInterpolation()


@dataclass
class MomentTensor2D:
    """src/shots/sources.jl:33-37."""
    Mxx: float
    Mzz: float
    Mxz: float


class MomentTensorSources:
    """src/shots/sources.jl:54-76."""

    def __init__(self, positions, tf, momtens: Sequence[MomentTensor2D], domfreq: float):
        positions = np.atleast_2d(np.asarray(positions, dtype=np.float64))
        tf = np.asarray(tf)
        assert positions.shape[0] > 0, "There must be at least one source!"
        assert positions.shape[0] == tf.shape[1], "Number of sources do not match between positions and time-functions!"
        assert len(momtens) == positions.shape[0], "Number of moment tensors must match number of sources!"
        self.positions, self.tf, self.momtens, self.domfreq = positions, tf, list(momtens), float(domfreq)


class ExternalForceSources:
    """src/shots/sources.jl:78-90: tf is (nt, ncomponents, nsrc)."""

    def __init__(self, positions, tf, domfreq: float):
        positions = np.atleast_2d(np.asarray(positions, dtype=np.float64))
        tf = np.asarray(tf)
        assert positions.shape[0] > 0, "There must be at least one source!"
        assert positions.shape[0] == tf.shape[2], "Number of sources do not match between positions and time-functions!"
        assert tf.shape[1] == positions.shape[1], "Number of components do not match between time-functions and positions!"
        self.positions, self.tf, self.domfreq = positions, tf, float(domfreq)


class VectorReceivers:
    """src/shots/receivers.jl:64-110: seismograms (nt, ndim, nrec)."""

    def __init__(self, positions, nt: int, ndim: int = 2):
        positions = np.atleast_2d(np.asarray(positions, dtype=np.float64))
        assert positions.shape[0] > 0, "There must be at least one receiver!"
        self.positions = positions
        self.seismograms = np.zeros((nt, ndim, positions.shape[0]), dtype=np.float64)


@dataclass
class MomentTensorShot:
    """src/shots/shot.jl:23-28."""
    srcs: MomentTensorSources
    recs: VectorReceivers


@dataclass
class ExternalForceShot:
    """src/shots/shot.jl:37-42."""
    srcs: ExternalForceSources
    recs: VectorReceivers


# ---------------------------------------------------------------------------
# Band-limited delta spreading (src/utils/utils.jl:62-214)
# ---------------------------------------------------------------------------
def _sinc(t: float) -> float:
    if t == 0.0:
        return 1.0
    if t == round(t):  # sinpi of an integer is exactly 0
        return 0.0
    return math.sin(math.pi * t) / (math.pi * t)


def _kaiser(x: float, r: float, beta: float) -> float:
    if not (-r <= x <= r):
        return 0.0
    return float(np.i0(beta * math.sqrt(1.0 - (x / r) ** 2)) / np.i0(beta))


def _findnearest(x, xstart, dx, n):
    xs = xstart + dx * np.arange(n)
    return int(np.argmin(np.abs(x - xs))) + 1


def coeffsinc1d(x0, dx, nx, r, beta, xstart, mirror, xbl, xbr):
    """coeffsinc1D (utils.jl:105-154): 1-based indices and weights, duplicates summed."""
    i0 = _findnearest(x0, xstart, dx, nx)
    kept = []
    for idx in range(i0 - r - 1, i0 + r + 2):
        xc = (idx - 1) * dx + xstart
        coe = _kaiser(xc - x0, r * dx, beta) * _sinc((xc - x0) / dx)
        if not abs(coe) <= 1e-15:
            kept.append((idx, coe))
    out: dict[int, float] = {}
    for idx, coe in kept:
        xc = (idx - 1) * dx + xstart
        if xc < xbl:
            idx = _findnearest(xbl + (xbl - xc), xstart, dx, nx)
            coe = -coe if mirror else coe
        elif xc > xbr:
            idx = _findnearest(xbr - (xc - xbr), xstart, dx, nx)
            coe = -coe if mirror else coe
        out[idx] = out.get(idx, 0.0) + coe
    return list(out.keys()), list(out.values())


def spread_positions(gridsize, spacing, positions, shift=(0.0, 0.0), mirror=False, r=4, beta=6.31,
                     freesurfposition="ongridbound"):
    """spread_positions (utils.jl:168-214): per position, (ij (npts, 2) 1-based, weights)."""
    if freesurfposition == "halfgridin":
        fs = [h / 2 for h in spacing]
    elif freesurfposition == "ongridbound":
        fs = [0.0 for _ in spacing]
    else:
        raise ValueError(f"spread_positions(): Wrong keyword argument freesurfposition {freesurfposition}")
    extent = [h * (n - 1) for n, h in zip(gridsize, spacing)]
    out = []
    for p in np.atleast_2d(positions):
        dims = [coeffsinc1d(p[d], spacing[d], gridsize[d], r, beta, shift[d], mirror, fs[d], extent[d])
                for d in range(len(gridsize))]
        (ix, cx), (iz, cz) = dims
        ij = np.array([[a, b] for b in iz for a in ix], dtype=np.int32).reshape(-1, 2)
        coef = np.array([x * z for z in cz for x in cx], dtype=np.float64)
        out.append((ij, coef))
    return out


def _table(entries):
    """[(ij, coef) per item] -> sw_point_table arrays."""
    offsets = np.zeros(len(entries) + 1, dtype=np.int32)
    for k, (ij, c) in enumerate(entries):
        offsets[k + 1] = offsets[k] + len(c)
    ij = np.ascontiguousarray(np.concatenate([np.asarray(e[0], np.int32).reshape(-1, 2) for e in entries])
                              if entries else np.zeros((0, 2), np.int32), dtype=np.int32)
    coef = np.ascontiguousarray(np.concatenate([np.asarray(e[1], np.float64).reshape(-1) for e in entries])
                                if entries else np.zeros(0), dtype=np.float32)
    return offsets, ij, coef


class ElasticIsoCPMLWaveSimulation:
    """build_wavesim product for the elastic isotropic C-PML case (ela_models.jl:177-420)."""

    def __init__(self, params: InputParametersElastic, matprop: ElasticIsoMaterialProperties, cpmlparams, *,
                 runparams, gradparams=None, gradient: bool = False, sincinterp: bool = True, device: int = 0):
        from .api import GradParameters, UniformFiniteDifferenceGrid, _BACKEND, _context
        nt, halo, freetop = params.ntimesteps, cpmlparams.halo, cpmlparams.freeboundtop
        assert halo >= 0, "CPML halo size must be non-negative!"
        ns_cpml = params.gridsize[:-1] if freetop else params.gridsize
        assert all(n >= 2 * halo + 3 for n in ns_cpml), \
            f"Number grid points in the dimensions with C-PML boundaries must be at least 2*halo+3 = {2 * halo + 3}!"
        if len(params.gridsize) != 2:
            raise NotImplementedError("Only elastic 2D is currently implemented.")
        if runparams.parall != _BACKEND:
            raise ValueError(f"No backend found for model of type ElasticIsoCPMLWaveSimulation and "
                             f"`parall =` {runparams.parall}. Argument `parall` must be {_BACKEND}.")
        if runparams.snapevery is not None:
            assert 1 <= runparams.snapevery < params.ntimesteps, \
                "Checkpointing frequency must be smaller than the number of timesteps!"
        self.params, self.cpmlparams, self.nt, self.dt = params, cpmlparams, nt, params.dt
        self.grid = UniformFiniteDifferenceGrid(params.gridsize, params.gridspacing)
        self.runparams, self.gradient, self.sincinterp = runparams, gradient, sincinterp
        self.gradparams = (gradparams or GradParameters()) if gradient else None
        self.matprop = copy.deepcopy(matprop)
        self.ctx = _context(device)
        prm = _lib.SwElasticParams()
        for d in range(2):
            prm.n[d] = params.gridsize[d]
            prm.h[d] = params.gridspacing[d]
        prm.dt, prm.halo, prm.rcoef, prm.freetop = params.dt, halo, float(cpmlparams.rcoef), int(freetop)
        prm.interp_rho = matprop.interp_method_ρ.code
        prm.interp_mu = matprop.interp_method_μ.code
        self._prm = prm
        gp = _lib.SwGradParams()
        if gradient:
            g = self.gradparams
            gp.check_freq, gp.mute_radius_src, gp.mute_radius_rec = g.check_freq, g.mute_radius_src, g.mute_radius_rec
            gp.compute_misfit = int(g.compute_misfit)
        self._h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.sw_elastic_create(self.ctx.h, ctypes.byref(prm), int(gradient), ctypes.byref(gp),
                                                      ctypes.byref(self._h)), "sw_elastic_create")

    def __del__(self):
        try:
            if self._h:
                self.ctx.lib.sw_elastic_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass

    # -- checks (ela_models.jl:94-141, checks.jl:43-94) ------------------------
    def vp(self, m=None):
        m = m or self.matprop
        return np.sqrt((np.asarray(m.λ) + 2.0 * np.asarray(m.μ)) / np.asarray(m.ρ))

    def check_matprop(self, m: ElasticIsoMaterialProperties):
        lam, mu, rho = (np.asarray(a) for a in (m.λ, m.μ, m.ρ))
        assert np.all(lam >= 0), "Lamè coefficient λ must be positive!"
        assert np.all(mu >= 0), "Lamè coefficient μ must be positive!"
        assert np.all(rho > 0), "Density must be positive!"
        vp = np.sqrt((lam + 2.0 * mu) / rho)
        assert vp.ndim == 2, "Material property dimensionality must be the same as the wavesim!"
        assert vp.shape == self.grid.size, \
            f"Material property number of grid points must be the same as the wavesim! \n {vp.shape}, {self.grid.size}"
        courant = float(np.max(vp)) * self.dt * math.sqrt(sum(1.0 / h ** 2 for h in self.grid.spacing)) * 7 / 6
        log.info("Courant number: %s", courant)
        if self.runparams.erroronCFL:
            assert courant < 1, f"Courant condition not satisfied! [{courant}]"
        elif courant > 1:
            warnings.warn(f"CFL condition not satisfied! [{courant}]")

    def set_matprop(self, m: ElasticIsoMaterialProperties):
        """update_matprop! + precomp_elaprop! (ela_models.jl:143-173; interpolation in the library)."""
        self.check_matprop(m)
        self.matprop = copy.deepcopy(m)
        arrs = [np.asfortranarray(a, dtype=np.float32) for a in (m.λ, m.μ, m.ρ)]
        if m.interp_method_ρ.code != self._prm.interp_rho or m.interp_method_μ.code != self._prm.interp_mu:
            raise ValueError("interpolation methods are fixed when the wavesim is built")
        self.ctx.check(self.ctx.lib.sw_elastic_set_material(self._h, *(a.ctypes.data for a in arrs)),
                       "sw_elastic_set_material")

    def check_numerics(self, shot):
        m = self.matprop
        vel_min = float(np.min(np.sqrt(np.asarray(m.μ) / np.asarray(m.ρ))))
        if vel_min == 0:
            vel_min = float(np.min(self.vp()))
        fmax = shot.srcs.domfreq * 2.0
        ppw = vel_min / (fmax * max(self.grid.spacing))
        min_ppw = self.runparams.minPPW
        log.info("Points per wavelength: %s", ppw)
        dh0 = round(vel_min / (min_ppw * fmax), 2) if min_ppw > 0 else float("inf")
        msg = (f"Not enough points per wavelength (assuming fmax = 2*domfreq)! \n [{round(ppw, 1)} instead of "
               f">= {min_ppw}]\n  Grid spacing should be <= {dh0}")
        if self.runparams.erroronPPW:
            assert ppw >= min_ppw, msg
        elif ppw < min_ppw:
            warnings.warn(msg)

    def check_positions(self, positions):
        positions = np.atleast_2d(positions)
        assert positions.shape[1] == 2, "Positions matrix do not match the dimension of the model!"
        for p in positions:
            for c in range(2):
                assert 0 <= p[c] <= self.grid.extent[c], f"Position {p} is not inside the grid!"
            for c in range(2):
                if c == 1 and self.cpmlparams.freeboundtop:
                    continue
                lo = self.grid.spacing[c] * self.cpmlparams.halo
                if not (lo <= p[c] <= self.grid.extent[c] - lo):
                    warnings.warn(f"Position {p} is inside the CPML region!")

    # -- per-shot host preprocessing -------------------------------------------
    def cpml_block(self, domfreq: float) -> np.ndarray:
        """init_bdc! (ela_init_bc.jl:7-40): [a, a_h, b, b_h] for x then z."""
        cp = self.cpmlparams
        vmax = float(np.max(self.vp())) if cp.vel_max is None else float(cp.vel_max)
        parts = []
        for d in range(2):
            parts += _lib.cpml_coefficients(vmax, self.dt, cp.halo, cp.rcoef, self.grid.spacing[d], domfreq,
                                            cp.freeboundtop and d == 1)
        return np.concatenate(parts).astype(np.float32)

    def possrcrec_scaletf(self, shot):
        """ela_models.jl:6-90: source and receiver point tables and tf / (dx dz)."""
        n, h = self.grid.size, self.grid.spacing
        mt = isinstance(shot, MomentTensorShot)
        if self.sincinterp:
            sp = lambda pos, sh, mir: spread_positions(n, h, pos, shift=sh, mirror=mir)  # noqa: E731
            if mt:
                src = [sp(shot.srcs.positions, (0.0, 0.0), True), sp(shot.srcs.positions, (h[0] / 2, h[1] / 2), True)]
            else:
                src = [sp(shot.srcs.positions, (h[0] / 2, 0.0), False), sp(shot.srcs.positions, (0.0, h[1] / 2), False)]
            rec = [sp(shot.recs.positions, (h[0] / 2, 0.0), False), sp(shot.recs.positions, (0.0, h[1] / 2), False)]
        else:
            from .api import nearest_grid_points
            ps = nearest_grid_points(shot.srcs.positions, h)
            pr = nearest_grid_points(shot.recs.positions, h)
            one = lambda idx: [(np.array([row], np.int32), np.ones(1)) for row in idx]  # noqa: E731
            src = [one(ps), one(ps)]
            rec = [one(pr), one(pr)]
        return src, rec, np.asarray(shot.srcs.tf, dtype=np.float64) / (h[0] * h[1])

    def _shot_structs(self, shots, misfits=None):
        keep, structs = [], (_lib.SwElasticShot * len(shots))()
        for k, shot in enumerate(shots):
            nt = shot.recs.seismograms.shape[0]
            nrec = shot.recs.positions.shape[0]
            src, rec, scal = self.possrcrec_scaletf(shot)
            mt = isinstance(shot, MomentTensorShot)
            assert scal.shape[0] >= nt, "source time functions shorter than the receivers' record"
            scal = np.asfortranarray(scal[:nt], dtype=np.float32)
            traces = np.zeros((nt, 2, nrec), dtype=np.float32, order="F")
            cp = self.cpml_block(shot.srcs.domfreq)
            st = structs[k]
            st.nt, st.kind, st.nsrc, st.nrec = nt, 0 if mt else 1, shot.srcs.positions.shape[0], nrec
            arrs = [scal, traces, cp]
            st.srctf, st.traces, st.cpml = scal.ctypes.data, traces.ctypes.data, cp.ctypes.data
            if mt:
                m3 = np.ascontiguousarray([[m.Mxx, m.Mzz, m.Mxz] for m in shot.srcs.momtens], dtype=np.float32)
                st.momtens = m3.ctypes.data
                arrs.append(m3)
            for t in range(2):
                for tab, tgt in ((src[t], st.src[t]), (rec[t], st.rec[t])):
                    off, ij, coef = _table(tab)
                    tgt.offsets, tgt.ij, tgt.coef = off.ctypes.data, ij.ctypes.data, coef.ctypes.data
                    arrs += [off, ij, coef]
            if misfits is not None:
                m = misfits[k]
                obs = np.asfortranarray(m.observed, dtype=np.float32)
                assert obs.shape == (nt, 2, nrec), "observed data shape must be (nt, 2, nrec)"
                st.observed = obs.ctypes.data
                arrs.append(obs)
                if getattr(m, "kind", 0) == 1:  # CCTSMisfit, per component trace
                    st.misfit_kind, st.misfit_dt = 1, m.dt
                diag = m.invcov_diagonal()
                if diag is not None:
                    diag = np.ascontiguousarray(diag, dtype=np.float32)
                    st.invcov_diag = diag.ctypes.data
                    arrs.append(diag)
                dense = m.invcov_dense()
                if dense is not None:
                    dense = np.asfortranarray(dense, dtype=np.float32)
                    st.invcov = dense.ctypes.data
                    arrs.append(dense)
                if m.windows:
                    win = np.ascontiguousarray(np.array(m.windows, dtype=np.int32).reshape(-1))
                    st.nwin, st.windows = len(m.windows), win.ctypes.data
                    arrs.append(win)
                sp_ = np.asfortranarray(shot.srcs.positions, dtype=np.float64)
                rp_ = np.asfortranarray(shot.recs.positions, dtype=np.float64)
                st.src_pos, st.rec_pos = sp_.ctypes.data, rp_.ctypes.data
                arrs += [sp_, rp_]
            keep.append((traces, arrs))
        return structs, keep

    def init_shots(self, shots):
        for shot in shots:
            self.check_numerics(shot)
            self.check_positions(shot.srcs.positions)
            self.check_positions(shot.recs.positions)

    def run_forward(self, shots):
        """Fills the seismograms; with RunParameters.snapevery returns, per shot,
        {it: {"ucur": [ux, uz], "σ": [σxx, σzz, σxz]}} (ela_forward.jl:74-78)."""
        self.init_shots(shots)
        structs, keep = self._shot_structs(shots)
        snapevery = self.runparams.snapevery
        nx, nz = self.grid.size
        shapes = [(nx - 1, nz), (nx, nz - 1), (nx, nz), (nx, nz), (nx - 1, nz - 1)]
        B = sum(a * b for a, b in shapes)
        if snapevery:
            bufs = [np.zeros((k[0].shape[0] // snapevery) * B, dtype=np.float32) for k in keep]
            ptrs = (ctypes.c_void_p * len(bufs))(*[b.ctypes.data for b in bufs])
            self.ctx.check(self.ctx.lib.sw_elastic_forward_snapshots(self._h, len(shots), structs, 0, snapevery,
                                                                     ptrs), "sw_elastic_forward_snapshots")
        else:
            self.ctx.check(self.ctx.lib.sw_elastic_forward(self._h, len(shots), structs, 0), "sw_elastic_forward")
        for shot, (traces, _) in zip(shots, keep):
            shot.recs.seismograms[...] = traces
        if not snapevery:
            return None
        out = []
        for b in bufs:
            d = {}
            for q, blk in enumerate(b.reshape(-1, B)):
                parts, o = [], 0
                for a_, b_ in shapes:
                    parts.append(blk[o:o + a_ * b_].reshape((a_, b_), order="F").copy())
                    o += a_ * b_
                d[(q + 1) * snapevery] = {"ucur": parts[:2], "σ": parts[2:]}
            out.append(d)
        return out

    def run_gradient(self, shots, misfits):
        assert self.gradient, "The wavesim object was not built for gradient computations. (Was `gradient=true` specified?)"
        assert len(misfits) == len(shots)
        self.init_shots(shots)
        structs, keep = self._shot_structs(shots, misfits)
        g = {k: np.zeros(self.grid.size, dtype=np.float64, order="F") for k in ("rho", "lambda", "mu")}
        misfit = np.zeros(1, dtype=np.float64)
        self.ctx.check(self.ctx.lib.sw_elastic_gradient(self._h, len(shots), structs, 0, g["rho"].ctypes.data,
                                                         g["lambda"].ctypes.data, g["mu"].ctypes.data,
                                                         misfit.ctypes.data), "sw_elastic_gradient")
        for shot, (traces, _) in zip(shots, keep):
            shot.recs.seismograms[...] = traces
        return g, float(misfit[0])
