"""Host-side mirror of SeismicWaves.jl's acoustic constant-density API over libswgb300.

The names, argument meanings and checks follow the reference (SeismicWaves.jl
v0.9.0); the Julia functions ending in ``!`` keep their behaviour (they fill
``shot.recs.seismograms``) under names without the ``!``:

    InputParametersAcoustic, CPMLBoundaryConditionParameters, RunParameters,
    GradParameters, VpAcousticCDMaterialProperties, ScalarSources,
    ScalarReceivers, ScalarShot, L2Misfit, CCTSMisfit, rickerstf, build_wavesim,
    swforward (swforward!), swmisfit (swmisfit!), swgradient (swgradient!)

Host logic kept from the reference: CFL and points-per-wavelength checks
(src/models/acoustic/acou_models.jl:5-38), position checks
(src/utils/checks.jl:43-94), C-PML coefficients per shot (init_bdc!,
src/models/acoustic/acou_init_bc.jl:7-40, computed by the library),
nearest-grid-point rounding and source scaling (possrcrec_scaletf,
src/models/acoustic/acou_forward.jl:6-20 / acou_models.jl:206-217) and the
L2 misfit (src/inversion/misfits/L2Misfit.jl:24-77).  The time stepping,
checkpointing, adjoint, correlation, misfit reduction and shot sum run on
the GPU, all shots of a call batched together.

Divergences from the reference, on purpose:
  * swmisfit sums the misfit of every shot (the reference's run_swmisfit!
    loop, src/apis/misfit.jl:97-101, only ever counts shot 1);
  * CPMLBoundaryConditionParameters.vel_max is honoured (the reference reads
    a non-existent field there, acou_init_bc.jl:16);
  * the wavefields are FP32 whatever the input precision; traces come back in
    the receivers' dtype and gradients as float64.
"""
from __future__ import annotations

import copy
import ctypes
import logging
import math
import warnings
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _lib

log = logging.getLogger("seismicwaves_gb300")

_BACKEND = "GB300"


def rickerstf(t, t0, f0):
    """Ricker wavelet (src/utils/utils.jl:6)."""
    a = (np.pi * f0 * (np.asarray(t) - t0)) ** 2
    return (1 - 2 * a) * np.exp(-a)


def gaussderivstf(t, t0, f0):
    """First derivative of a Gaussian (src/utils/utils.jl:13)."""
    t = np.asarray(t)
    return (t - t0) * np.exp(-((np.pi * f0 * (t - t0)) ** 2))


def gaussstf(t, t0, f0):
    """Gaussian (src/utils/utils.jl:20)."""
    return -np.exp(-((np.pi * f0 * (np.asarray(t) - t0)) ** 2)) / (2 * (np.pi * f0) ** 2)


@dataclass
class CPMLBoundaryConditionParameters:
    """src/models/bdc_params.jl:16-25."""
    halo: int = 20
    rcoef: float = 0.0001
    freeboundtop: bool = True
    vel_max: float | None = None


class InputParametersAcoustic:
    """src/models/acoustic/acou_params.jl:9-35."""

    def __init__(self, ntimesteps: int, dt: float, gridsize: Sequence[int], gridspacing: Sequence[float],
                 boundcond: CPMLBoundaryConditionParameters):
        gridsize = tuple(int(n) for n in gridsize)
        gridspacing = tuple(float(h) for h in gridspacing)
        N = len(gridsize)
        assert N <= 3, "Dimensionality must be less than or equal to 3!"
        assert len(gridspacing) == N
        assert all(n > 0 for n in gridsize), "All numbers of grid points must be positive!"
        assert all(h > 0 for h in gridspacing), "All grid spacings must be positive!"
        assert ntimesteps > 0, "Number of timesteps must be positive!"
        assert dt > 0, "Timestep size must be positive!"
        self.ntimesteps, self.dt = int(ntimesteps), float(dt)
        self.gridsize, self.gridspacing, self.boundcond = gridsize, gridspacing, boundcond


@dataclass
class VpAcousticCDMaterialProperties:
    """src/models/acoustic/acou_params.jl:9-12."""
    vp: np.ndarray


class ScalarSources:
    """src/shots/sources.jl:8-26."""

    def __init__(self, positions, tf, domfreq):
        positions = np.atleast_2d(np.asarray(positions))
        tf = np.asarray(tf)
        if tf.ndim == 1:
            tf = tf.reshape(-1, 1)
        assert positions.shape[0] > 0, "There must be at least one source!"
        assert positions.shape[0] == tf.shape[1], \
            "Number of sources do not match between positions and time-functions!"
        self.positions, self.tf, self.domfreq = positions, tf, float(domfreq)


class ScalarReceivers:
    """src/shots/receivers.jl:8-57."""

    def __init__(self, positions, nt: int):
        positions = np.atleast_2d(np.asarray(positions))
        assert positions.shape[0] > 0, "There must be at least one receiver!"
        dtype = positions.dtype if np.issubdtype(positions.dtype, np.floating) else np.float64
        self.positions = positions
        self.seismograms = np.zeros((int(nt), positions.shape[0]), dtype=dtype, order="F")


@dataclass
class ScalarShot:
    """src/shots/shot.jl:9-16."""
    srcs: ScalarSources
    recs: ScalarReceivers


class L2Misfit:
    """src/inversion/misfits/L2Misfit.jl:2-20.

    ``invcov`` may be None (identity), a vector (its diagonal) or a square
    matrix (applied on the GPU by the library's own tiled FP32 product when it
    has off-diagonal terms).
    """

    def __init__(self, observed=None, invcov=None, windows: Sequence[tuple[int, int]] = ()):
        observed = np.zeros((0, 0)) if observed is None else np.asarray(observed)
        if observed.ndim not in (2, 3):
            raise ValueError("Observed data must be a 2D or 3D array!")
        nt = observed.shape[0]
        if invcov is not None:
            invcov = np.asarray(invcov)
            if invcov.ndim == 2:
                assert invcov.shape[0] == invcov.shape[1], "Inverse covariance matrix must be square!"
            assert invcov.shape[0] == nt, "Size of inverse covariance matrix must match the number of timesteps!"
        windows = [(int(a), int(b)) for a, b in windows]
        assert all(1 <= a <= b <= nt for a, b in windows), \
            "Windows indices must be between 1 and maximum number of timesteps!"
        self.observed = observed.copy()
        self.invcov = invcov
        self.windows = windows

    def invcov_diagonal(self):
        """Diagonal of C^-1 (None = identity or a non-diagonal matrix, see invcov_dense)."""
        ic = self.invcov
        if ic is None:
            return None
        if ic.ndim == 1:
            return ic
        d = np.diag(ic)
        return d if np.count_nonzero(ic - np.diag(d)) == 0 else None

    def invcov_dense(self):
        """C^-1 as a dense (nt, nt) matrix when it has off-diagonal terms, else None."""
        ic = self.invcov
        if ic is None or ic.ndim == 1 or self.invcov_diagonal() is not None:
            return None
        return ic

    def _masked_residuals(self, seismograms):
        res = np.asarray(seismograms, dtype=np.float64) - self.observed
        if self.windows:
            mask = np.zeros(res.shape[0])
            for a, b in self.windows:
                mask[a - 1:b] = 1.0
            res = mask.reshape((-1,) + (1,) * (res.ndim - 1)) * res
        return res

    def _apply_invcov(self, res):
        """C^-1 applied along time; for (nt, ncomp, nrec) traces per component (L2Misfit.jl:79-95)."""
        if self.invcov is None:
            return res
        if self.invcov.ndim == 1:
            return self.invcov.reshape((-1,) + (1,) * (res.ndim - 1)) * res
        if res.ndim == 3:
            return np.einsum("tu,ucr->tcr", self.invcov, res)
        return self.invcov @ res

    def calcmisfit(self, recs) -> float:
        """L2Misfit.jl:24-62: 1/2 r' C^-1 r (summed over components for vector receivers)."""
        res = self._masked_residuals(recs.seismograms)
        return float(np.sum(res * self._apply_invcov(res)) / 2)

    def dchi_du(self, recs):
        """L2Misfit.jl:64-95: C^-1 r."""
        return self._apply_invcov(self._masked_residuals(recs.seismograms))


class CCTSMisfit:
    """src/inversion/misfits/CCTSMisfit.jl:1-15: cross-correlation time-shift misfit.

    Per trace, dtau = (first index of max |xcorr(observed, synthetic)| - (nt - 1)) * dt
    with DSP.jl's xcorr (conv(u, reverse(v)), 1-based index k holding
    sum_i u[i] v[i - (k - nt)]); the misfit is sum dtau^2 / 2 and dchi/du =
    dtau / N * ds/dt (CCTSMisfit.jl:17-80).  ``std`` is stored, as in the
    reference, and not used.  The gradient evaluates it on the GPU (k_ccts);
    these host versions serve swmisfit and checks.
    """
    kind = 1

    def __init__(self, dt: float, std: float = 1.0, observed=None):
        observed = np.zeros((0, 0)) if observed is None else np.asarray(observed)
        if observed.ndim not in (2, 3):
            raise ValueError("Observed data must be a 2D or 3D array!")
        assert dt > 0, "Timestep size must be positive!"
        assert std > 0, "Standard deviation must be positive!"
        self.dt, self.std = float(dt), float(std)
        self.observed = observed.copy()
        self.windows = []
        self.invcov = None

    def invcov_diagonal(self):
        return None

    def invcov_dense(self):
        return None

    def _traces(self, seismograms):
        s = np.asarray(seismograms, dtype=np.float64)
        o = np.asarray(self.observed, dtype=np.float64)
        nt = s.shape[0]
        return s.reshape(nt, -1, order="F"), o.reshape(nt, -1, order="F"), s.shape

    def _dtau(self, obs, syn):
        # numpy's correlate(a, v, "full")[k0] = sum_n a[n + k0 - (nt - 1)] v[n] = DSP xcorr(a, v)[k0 + 1]
        c = np.correlate(obs, syn, "full")
        return (int(np.argmax(np.abs(c))) + 1 - (len(syn) - 1)) * self.dt

    def calcmisfit(self, recs) -> float:
        s, o, _ = self._traces(recs.seismograms)
        return float(sum(self._dtau(o[:, r], s[:, r]) ** 2 / 2 for r in range(s.shape[1])))

    def dchi_du(self, recs):
        s, o, shape = self._traces(recs.seismograms)
        nt, dt = s.shape[0], self.dt
        ds = np.zeros_like(s)
        ds[1:-1] = (s[2:] - s[:-2]) / (2 * dt)
        ds[0] = (s[1] - 0) / (2 * dt)
        out = np.zeros_like(s)
        for r in range(s.shape[1]):
            dtau = self._dtau(o[:, r], s[:, r])
            y = ds[:, r] ** 2
            norm = float(np.sum(dt * (y[:-1] + y[1:]) / 2))
            out[:, r] = dtau / norm * ds[:, r]
        return out.reshape(shape, order="F")


@dataclass
class RunParameters:
    """src/models/genparameters.jl:25-46 (parall selects the backend; only :GB300 here).

    compensated (an addition of this backend, False by default): the forward
    passes of the acoustic simulations (constant density: p and d; variable
    density: p, vx and vz) keep their state as pairs of FP32 numbers and form
    the material factors from the FP64 model (sw_wavesim_set_precision /
    sw_wavesim_set_vp64, sw_acoustic_vd_set_precision /
    sw_acoustic_vd_set_material64): traces and misfit within ~1e-8 of an
    FP64 run at thousands of steps instead of ~1e-6, at several times the
    forward's cost.
    """
    parall: str = _BACKEND
    snapevery: int | None = None
    infoevery: int | None = None
    logger: logging.Logger | None = None
    erroronCFL: bool = True
    minPPW: int = 10
    erroronPPW: bool = True
    compensated: bool = False

    def __post_init__(self):
        assert self.minPPW >= 0


@dataclass
class GradParameters:
    """src/models/genparameters.jl:63-79.

    snapshot_bf16 (an addition of this backend, 0 by default): 1 keeps the
    acoustic recompute buffer (the second time differences between
    checkpoints) in BF16 -- half its memory and traffic, gradient within 1e-3
    instead of 1e-5 of the FP64 result; 2 also keeps the checkpoints' (p, d)
    as per-snapshot-scaled BF16 (a few 1e-3).
    """
    mute_radius_src: int = 0
    mute_radius_rec: int = 0
    compute_misfit: bool = False
    check_freq: int = 1
    snapshot_bf16: int = 0

    def __post_init__(self):
        assert self.check_freq > 0


@dataclass
class UniformFiniteDifferenceGrid:
    """src/utils/grids.jl:1-17 (size, spacing, extent)."""
    size: tuple
    spacing: tuple
    extent: tuple = field(init=False)

    def __post_init__(self):
        self.extent = tuple(h * (n - 1) for n, h in zip(self.size, self.spacing))


def nearest_grid_points(positions, spacing) -> np.ndarray:
    """round(pos/h + 1, RoundNearestTiesUp), 1-based int32 (acou_models.jl:206-217)."""
    positions = np.atleast_2d(np.asarray(positions, dtype=np.float64))
    idx = np.floor(positions / np.asarray(spacing, dtype=np.float64) + 1 + 0.5)
    return np.asfortranarray(idx.astype(np.int32))


def scale_srctf(tf, possrcs, vp, spacing, dt) -> np.ndarray:
    """tf ./ prod(h) .* dt^2, times vp(src)^2 per source (acou_forward.jl:6-20); float32 result."""
    vp = np.asarray(vp, dtype=np.float64)
    scal = np.asarray(tf, dtype=np.float64) / float(np.prod(spacing)) * dt ** 2
    scal = np.array(scal, copy=True)
    for s in range(scal.shape[1]):
        scal[:, s] *= vp[tuple(np.asarray(possrcs[s]) - 1)] ** 2
    return np.asfortranarray(scal.astype(np.float32))


def courant_number(vp, dt, spacing) -> float:
    """check_courant_condition (acou_models.jl:5-16)."""
    return float(np.max(vp)) * dt * math.sqrt(sum(1.0 / h ** 2 for h in spacing))


def points_per_wavelength(vp, spacing, domfreq) -> float:
    """check_numerics (acou_models.jl:18-38): vmin / (2 f0 hmax)."""
    return float(np.min(vp)) / (2.0 * domfreq * max(spacing))


_context_cache: dict[int, _lib.Context] = {}


def _context(device: int = 0) -> _lib.Context:
    if device not in _context_cache:
        _context_cache[device] = _lib.Context(device)
    return _context_cache[device]


class AcousticCDCPMLWaveSimulation:
    """build_wavesim product for the acoustic CD C-PML case (acou_models.jl:68-202).

    Holds the device-side simulation (sw_wavesim); device memory for the shots
    is allocated on first use and reused by later calls.
    """

    def __init__(self, params: InputParametersAcoustic, matprop: VpAcousticCDMaterialProperties,
                 cpmlparams: CPMLBoundaryConditionParameters, *, runparams: RunParameters,
                 gradparams: GradParameters | None, gradient: bool = False, device: int = 0):
        nt, halo, freetop = params.ntimesteps, cpmlparams.halo, cpmlparams.freeboundtop
        assert halo >= 0, "CPML halo size must be non-negative!"
        ns_cpml = params.gridsize[:-1] if freetop else params.gridsize
        assert all(n >= 2 * halo + 3 for n in ns_cpml), \
            f"Number grid points in the dimensions with C-PML boundaries must be at least 2*halo+3 = {2 * halo + 3}!"
        N = len(params.gridsize)
        if N not in (2, 3):
            raise NotImplementedError("the GB300 backend covers the 2D and 3D acoustic constant-density path")
        if runparams.parall != _BACKEND:
            raise ValueError(f"No backend found for model of type AcousticCDCPMLWaveSimulation and "
                             f"`parall =` {runparams.parall}. Argument `parall` must be {_BACKEND}.")
        if runparams.snapevery is not None:
            assert 1 <= runparams.snapevery < nt, "Checkpointing frequency must be smaller than the number of timesteps!"
        if runparams.infoevery is not None:
            assert 1 <= runparams.infoevery <= nt, "Infoevery parameter must be positive and less then nt!"
        self.params, self.cpmlparams, self.nt, self.dt = params, cpmlparams, nt, params.dt
        self.grid = UniformFiniteDifferenceGrid(params.gridsize, params.gridspacing)
        self.runparams, self.gradparams, self.gradient = runparams, gradparams, gradient
        self.matprop = copy.deepcopy(matprop)
        self.ctx = _context(device)
        prm = _lib.SwAcousticParams()
        prm.ndim = N
        for d in range(N):
            prm.n[d] = params.gridsize[d]
            prm.h[d] = params.gridspacing[d]
        prm.dt, prm.halo, prm.rcoef, prm.freetop = params.dt, halo, float(cpmlparams.rcoef), int(freetop)
        gp = _lib.SwGradParams()
        if gradient:
            g = gradparams or GradParameters()
            gp.check_freq, gp.mute_radius_src, gp.mute_radius_rec = g.check_freq, g.mute_radius_src, g.mute_radius_rec
            gp.compute_misfit = int(g.compute_misfit)
            gp.snapshot_bf16 = int(g.snapshot_bf16)
        self._h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.sw_wavesim_create(self.ctx.h, ctypes.byref(prm), int(gradient),
                                                      ctypes.byref(gp), ctypes.byref(self._h)),
                       "sw_wavesim_create")
        if runparams.compensated:
            self.ctx.check(self.ctx.lib.sw_wavesim_set_precision(self._h, 1), "sw_wavesim_set_precision")

    def __del__(self):
        try:
            if self._h:
                self.ctx.lib.sw_wavesim_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass

    # -- checks (acou_models.jl:5-51, checks.jl:43-94) -------------------------
    def check_matprop(self, matprop: VpAcousticCDMaterialProperties):
        vp = np.asarray(matprop.vp)
        assert vp.ndim == len(self.grid.size), "Material property dimensionality must be the same as the wavesim!"
        assert vp.shape == self.grid.size, (
            f"Material property number of grid points must be the same as the wavesim! \n {vp.shape}, "
            f"{self.grid.size}")
        assert np.all(vp > 0), "Pressure velocity material property must be positive!"
        courant = courant_number(vp, self.dt, self.grid.spacing)
        log.info("Courant number: %s", courant)
        if self.runparams.erroronCFL:
            assert courant < 1, f"Courant condition not satisfied! [{courant}]"
        elif courant > 1:
            warnings.warn(f"CFL condition not satisfied! [{courant}]")

    def set_matprop(self, matprop: VpAcousticCDMaterialProperties):
        """set_wavesim_matprop! (src/apis/utils.jl:3-8)."""
        self.check_matprop(matprop)
        self.matprop = VpAcousticCDMaterialProperties(np.array(matprop.vp, copy=True))
        if self.runparams.compensated:  # fact from the FP64 model
            vp64 = np.asfortranarray(matprop.vp, dtype=np.float64)
            self.ctx.check(self.ctx.lib.sw_wavesim_set_vp64(self._h, vp64.ctypes.data, 0), "sw_wavesim_set_vp64")
        else:
            vp32 = np.asfortranarray(matprop.vp, dtype=np.float32)
            self.ctx.check(self.ctx.lib.sw_wavesim_set_vp(self._h, vp32.ctypes.data, 0), "sw_wavesim_set_vp")

    def check_numerics(self, shot: ScalarShot):
        vel_min = float(np.min(self.matprop.vp))
        fmax = shot.srcs.domfreq * 2.0
        ppw = points_per_wavelength(self.matprop.vp, self.grid.spacing, shot.srcs.domfreq)
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
        N = len(self.grid.size)
        assert positions.shape[1] == N, "Positions matrix do not match the dimension of the model!"
        for p in positions:
            for c in range(N):
                assert 0 <= p[c] <= self.grid.extent[c], f"Position {p} is not inside the grid!"
            for c in range(N):
                if c == N - 1 and self.cpmlparams.freeboundtop:
                    continue
                lo = self.grid.spacing[c] * self.cpmlparams.halo
                if not (lo <= p[c] <= self.grid.extent[c] - lo):
                    warnings.warn(f"Position {p} is inside the CPML region!")

    # -- per-shot host preprocessing -------------------------------------------
    def cpml_block(self, domfreq: float, fp64: bool = False) -> np.ndarray:
        """init_bdc!: this shot's coefficients, [a, a_h, b, b_h] per axis (FP32, or FP64 for the
        compensated forward)."""
        cp = self.cpmlparams
        vmax = float(np.max(self.matprop.vp)) if cp.vel_max is None else float(cp.vel_max)
        N = len(self.grid.size)
        coeffs = _lib.cpml_coefficients64 if fp64 else _lib.cpml_coefficients
        parts = []
        for d in range(N):
            parts += coeffs(vmax, self.dt, cp.halo, cp.rcoef, self.grid.spacing[d], domfreq,
                            cp.freeboundtop and d == N - 1)
        return np.concatenate(parts).astype(np.float64 if fp64 else np.float32)

    def find_nearest_grid_points(self, positions) -> np.ndarray:
        return nearest_grid_points(positions, self.grid.spacing)

    def possrcrec_scaletf(self, shot: ScalarShot):
        """acou_forward.jl:6-20: indices and tf * dt^2 * vp(src)^2 / prod(h)."""
        possrcs = nearest_grid_points(shot.srcs.positions, self.grid.spacing)
        posrecs = nearest_grid_points(shot.recs.positions, self.grid.spacing)
        return possrcs, posrecs, scale_srctf(shot.srcs.tf, possrcs, self.matprop.vp, self.grid.spacing, self.dt)

    def _shot_structs(self, shots, misfits=None):
        keep, structs = [], (_lib.SwAcousticShot * len(shots))()
        for k, shot in enumerate(shots):
            nt = shot.recs.seismograms.shape[0]
            assert shot.srcs.tf.shape[0] >= nt, "source time functions shorter than the receivers' record"
            possrcs, posrecs, scal = self.possrcrec_scaletf(shot)
            scal = np.asfortranarray(scal[:nt])
            traces = np.zeros((nt, posrecs.shape[0]), dtype=np.float32, order="F")
            cp = self.cpml_block(shot.srcs.domfreq)
            st = structs[k]
            st.nt, st.nsrc, st.nrec = nt, possrcs.shape[0], posrecs.shape[0]
            st.src_idx, st.rec_idx = possrcs.ctypes.data, posrecs.ctypes.data
            st.srctf, st.traces, st.cpml = scal.ctypes.data, traces.ctypes.data, cp.ctypes.data
            arrs = [possrcs, posrecs, scal, traces, cp]
            if self.runparams.compensated:
                cp64 = self.cpml_block(shot.srcs.domfreq, fp64=True)
                st.cpml64 = cp64.ctypes.data
                arrs.append(cp64)
            if misfits is not None:
                m = misfits[k]
                obs = np.asfortranarray(m.observed, dtype=np.float32)
                assert obs.shape == (nt, posrecs.shape[0]), "observed data shape must be (nt, nrec)"
                st.observed = obs.ctypes.data
                arrs.append(obs)
                if isinstance(m, CCTSMisfit):
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
                sp = np.asfortranarray(shot.srcs.positions, dtype=np.float64)
                rp = np.asfortranarray(shot.recs.positions, dtype=np.float64)
                st.src_pos, st.rec_pos = sp.ctypes.data, rp.ctypes.data
                arrs += [sp, rp]
            keep.append((traces, arrs))
        return structs, keep

    def init_shots(self, shots):
        for shot in shots:
            self.check_numerics(shot)
            self.check_positions(shot.srcs.positions)
            self.check_positions(shot.recs.positions)

    def run_forward(self, shots):
        """Fills the seismograms; with RunParameters.snapevery returns, per shot, the
        reference's snapshot Dict {it: {"pcur": p[it]}} (run_swforward!, forward.jl:90-114)."""
        self.init_shots(shots)
        structs, keep = self._shot_structs(shots)
        snapevery = self.runparams.snapevery
        if snapevery:
            npts = int(np.prod(self.grid.size))
            bufs = [np.zeros((k[0].shape[0] // snapevery) * npts, dtype=np.float32) for k in keep]
            ptrs = (ctypes.c_void_p * len(bufs))(*[b.ctypes.data for b in bufs])
            self.ctx.check(self.ctx.lib.sw_acoustic_forward_snapshots(self._h, len(shots), structs, 0, snapevery,
                                                                      ptrs), "sw_acoustic_forward_snapshots")
        else:
            self.ctx.check(self.ctx.lib.sw_acoustic_forward(self._h, len(shots), structs, 0), "sw_acoustic_forward")
        for shot, (traces, _) in zip(shots, keep):
            shot.recs.seismograms[...] = traces
        if not snapevery:
            return None
        out = []
        for b in bufs:
            snaps = b.reshape(-1, npts)
            out.append({(q + 1) * snapevery: {"pcur": snaps[q].reshape(self.grid.size, order="F").copy()}
                        for q in range(snaps.shape[0])})
        return out

    def run_gradient(self, shots, misfits):
        assert self.gradient, "The wavesim object was not built for gradient computations. (Was `gradient=true` specified?)"
        assert len(misfits) == len(shots)
        self.init_shots(shots)
        structs, keep = self._shot_structs(shots, misfits)
        grad = np.zeros(self.grid.size, dtype=np.float64, order="F")
        misfit = np.zeros(1, dtype=np.float64)
        self.ctx.check(self.ctx.lib.sw_acoustic_gradient(self._h, len(shots), structs, 0, grad.ctypes.data,
                                                          misfit.ctypes.data), "sw_acoustic_gradient")
        for shot, (traces, _) in zip(shots, keep):
            shot.recs.seismograms[...] = traces
        return grad, float(misfit[0])

    def set_tuning(self, tz: int = 0, variant: int = 0):
        self.ctx.check(self.ctx.lib.sw_wavesim_set_tuning(self._h, int(tz), int(variant)), "sw_wavesim_set_tuning")


def _check_sim_consistency(matprop, shots):
    """src/utils/checks.jl:2-41 for the acoustic CD / VD and the elastic isotropic 2D cases."""
    from . import elastic as E
    from . import vd as V
    if isinstance(matprop, V.VpRhoAcousticVDMaterialProperties):
        for s in shots:
            if not (isinstance(s.srcs, ScalarSources) and isinstance(s.recs, ScalarReceivers)):
                raise TypeError("Types of shots are inconsistent.")
        return
    if isinstance(matprop, E.ElasticIsoMaterialProperties):
        kinds = {type(s) for s in shots}
        if len(kinds) != 1:
            raise TypeError("Types of shots are inconsistent.")
        for s in shots:
            ok = (isinstance(s, E.MomentTensorShot) and isinstance(s.srcs, E.MomentTensorSources)) or \
                 (isinstance(s, E.ExternalForceShot) and isinstance(s.srcs, E.ExternalForceSources))
            if not (ok and isinstance(s.recs, E.VectorReceivers)):
                raise TypeError("Types of WaveSimulation, MaterialProperties and Sources/Receivers are inconsistent")
        return
    if not isinstance(matprop, VpAcousticCDMaterialProperties):
        raise TypeError("Types of WaveSimulation, MaterialProperties and Sources/Receivers are inconsistent")
    for s in shots:
        if not (isinstance(s.srcs, ScalarSources) and isinstance(s.recs, ScalarReceivers)):
            raise TypeError("Types of shots are inconsistent.")


def build_wavesim(params, matprop, *, runparams: RunParameters, gradparams: GradParameters | None = None,
                  gradient: bool | None = None, device: int = 0, sincinterp: bool = True):
    """src/apis/build.jl:18-90: AcousticCDCPMLWaveSimulation, AcousticVDStaggeredCPMLWaveSimulation or
    ElasticIsoCPMLWaveSimulation."""
    from . import elastic as E
    if gradparams is None and gradient:
        gradparams = GradParameters()
    elif gradparams is not None:
        assert gradient is True, \
            "build_wavesim(...) specifies GradParameters, however, gradient keyword argument is set to false."
    if not isinstance(params.boundcond, CPMLBoundaryConditionParameters):
        raise NotImplementedError("the GB300 backend implements C-PML boundaries")
    if runparams.parall == "threadpersrc":
        raise ValueError("`parall = :threadpersrc` is a CPU-threads mode; the GB300 backend batches shots itself")
    if isinstance(params, E.InputParametersElastic):
        if not isinstance(matprop, E.ElasticIsoMaterialProperties):
            raise TypeError("elastic input parameters need ElasticIsoMaterialProperties")
        return E.ElasticIsoCPMLWaveSimulation(params, matprop, params.boundcond, runparams=runparams,
                                              gradparams=gradparams, gradient=bool(gradient), sincinterp=sincinterp,
                                              device=device)
    from . import vd as V
    if isinstance(matprop, V.VpRhoAcousticVDMaterialProperties):
        return V.AcousticVDStaggeredCPMLWaveSimulation(params, matprop, params.boundcond, runparams=runparams,
                                                       gradparams=gradparams, gradient=bool(gradient), device=device)
    if not isinstance(matprop, VpAcousticCDMaterialProperties):
        raise NotImplementedError("the GB300 backend implements the acoustic constant- and variable-density "
                                  "and the elastic isotropic simulations")
    return AcousticCDCPMLWaveSimulation(params, matprop, params.boundcond, runparams=runparams,
                                        gradparams=gradparams, gradient=bool(gradient), device=device)


def _prepare(params_or_wavesim, matprop, runparams, gradient, gradparams=None):
    from . import elastic as E
    if isinstance(params_or_wavesim, (AcousticCDCPMLWaveSimulation, E.ElasticIsoCPMLWaveSimulation)):
        ws = params_or_wavesim
        if gradient and not ws.gradient:
            raise AssertionError("The wavesim object was not built for gradient computations. "
                                 "(Was `gradient=true` specified?)")
        return ws
    return build_wavesim(params_or_wavesim, matprop, runparams=runparams or RunParameters(),
                         gradparams=gradparams if gradient else None, gradient=gradient)


def swforward(params_or_wavesim, matprop: VpAcousticCDMaterialProperties, shots: Sequence[ScalarShot], *,
              runparams: RunParameters | None = None):
    """swforward! (src/apis/forward.jl:24-66): fills shot.recs.seismograms of every shot; with
    RunParameters.snapevery returns the snapshots of every shot (a list of Dicts {it: fields})."""
    ws = _prepare(params_or_wavesim, matprop, runparams, False)
    _check_sim_consistency(matprop, shots)
    ws.set_matprop(matprop)
    return ws.run_forward(list(shots))


def swmisfit(params_or_wavesim, matprop: VpAcousticCDMaterialProperties, shots: Sequence[ScalarShot],
             misfit: Sequence[L2Misfit], *, runparams: RunParameters | None = None) -> float:
    """swmisfit! (src/apis/misfit.jl:26-104): forward, then the summed misfit of every shot."""
    swforward(params_or_wavesim, matprop, shots, runparams=runparams)
    return float(sum(m.calcmisfit(s.recs) for s, m in zip(shots, misfit)))


def swgradient(params_or_wavesim, matprop: VpAcousticCDMaterialProperties, shots: Sequence[ScalarShot],
               misfit: Sequence[L2Misfit], *, runparams: RunParameters | None = None,
               gradparams: GradParameters | None = None):
    """swgradient! (src/apis/gradient.jl:31-136).

    Acoustic CD: returns {"vp": gradient}; acoustic VD: {"vp": , "rho": }; elastic: {"rho": , "lambda": , "mu": }
    (float64), with the summed misfit as a second value when
    gradparams.compute_misfit is true.
    """
    gradparams = gradparams or GradParameters()
    ws = _prepare(params_or_wavesim, matprop, runparams, True, gradparams)
    _check_sim_consistency(matprop, shots)
    ws.set_matprop(matprop)
    grad, msf = ws.run_gradient(list(shots), list(misfit))
    g = ws.gradparams or gradparams
    out = grad if isinstance(grad, dict) else {"vp": grad}
    return (out, msf) if g.compute_misfit else out
