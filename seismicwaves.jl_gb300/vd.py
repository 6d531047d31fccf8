"""Host-side mirror of SeismicWaves.jl's variable-density acoustic API over libswgb300.

    VpRhoAcousticVDMaterialProperties, AcousticVDStaggeredCPMLWaveSimulation

``build_wavesim`` / ``swforward`` / ``swmisfit`` / ``swgradient`` (module
``api``) dispatch here when the material properties carry a density, as
build_concrete_wavesim does in the reference (src/apis/build.jl:60-72).

Host logic kept from the reference (SeismicWaves.jl v0.9.0): the material
checks and the CFL condition with the 7/6 factor of the 4th-order stencil
(src/models/acoustic/acou_models.jl:240-281), the points-per-wavelength
check, the position checks, the per-shot C-PML coefficients (init_bdc!,
acou_init_bc.jl:7-40), nearest-grid-point rounding and the VD source scaling
tf * dt * vp(src)^2 rho(src) / prod(h) (acou_forward.jl:66-80).  The time
stepping, checkpointing, adjoint, correlations, back-interpolation, muting
and the vp / rho chain rule run on the GPU (sw_acoustic_vd_*), all shots of a
call batched together.  The backend covers the 2D simulation.
"""
from __future__ import annotations

import copy
import ctypes
import logging
import math
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .api import (AcousticCDCPMLWaveSimulation, CPMLBoundaryConditionParameters, GradParameters,
                  InputParametersAcoustic, RunParameters, ScalarShot, UniformFiniteDifferenceGrid, _BACKEND,
                  _context, nearest_grid_points)
from .elastic import ArithmeticAverageInterpolation

log = logging.getLogger("seismicwaves_gb300")


@dataclass
class VpRhoAcousticVDMaterialProperties:
    """acou_material_properties.jl:15-45: vp, rho and the interpolation of 1/rho to the half points."""
    vp: np.ndarray
    rho: np.ndarray
    interp_method: object = field(default_factory=ArithmeticAverageInterpolation)


def vd_courant_number(vp, dt, spacing) -> float:
    """check_courant_condition of the VD simulation (acou_models.jl:240-251)."""
    return float(np.max(vp)) * dt * math.sqrt(sum(1.0 / h ** 2 for h in spacing)) * 7 / 6


def scale_srctf_vd(tf, possrcs, vp, rho, spacing, dt) -> np.ndarray:
    """tf ./ prod(h) .* dt, times vp(src)^2 rho(src) per source (acou_forward.jl:66-80); float32 result."""
    vp = np.asarray(vp, dtype=np.float64)
    rho = np.asarray(rho, dtype=np.float64)
    scal = np.array(np.asarray(tf, dtype=np.float64) / float(np.prod(spacing)) * dt, copy=True)
    for s in range(scal.shape[1]):
        ij = tuple(np.asarray(possrcs[s]) - 1)
        scal[:, s] *= vp[ij] ** 2 * rho[ij]
    return np.asfortranarray(scal.astype(np.float32))


class AcousticVDStaggeredCPMLWaveSimulation(AcousticCDCPMLWaveSimulation):
    """build_wavesim product for the acoustic VD C-PML case (acou_models.jl:311-454).

    Holds the device-side simulation (sw_acoustic_vd); shares the position,
    numerics and C-PML host logic with the constant-density simulation.
    """

    def __init__(self, params: InputParametersAcoustic, matprop: VpRhoAcousticVDMaterialProperties,
                 cpmlparams: CPMLBoundaryConditionParameters, *, runparams: RunParameters,
                 gradparams: GradParameters | None, gradient: bool = False, device: int = 0):
        nt, halo, freetop = params.ntimesteps, cpmlparams.halo, cpmlparams.freeboundtop
        assert halo >= 0, "CPML halo size must be non-negative!"
        ns_cpml = params.gridsize[:-1] if freetop else params.gridsize
        assert all(n >= 2 * halo + 3 for n in ns_cpml), \
            f"Number grid points in the dimensions with C-PML boundaries must be at least 2*halo+3 = {2 * halo + 3}!"
        if len(params.gridsize) != 2:
            raise NotImplementedError("the GB300 backend covers the 2D variable-density acoustic path")
        if runparams.parall != _BACKEND:
            raise ValueError(f"No backend found for model of type AcousticVDStaggeredCPMLWaveSimulation and "
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
        prm.ndim = 2
        for d in range(2):
            prm.n[d] = params.gridsize[d]
            prm.h[d] = params.gridspacing[d]
        prm.n[2], prm.h[2] = 1, 1.0
        prm.dt, prm.halo, prm.rcoef, prm.freetop = params.dt, halo, float(cpmlparams.rcoef), int(freetop)
        gp = _lib.SwGradParams()
        if gradient:
            g = gradparams or GradParameters()
            if g.snapshot_bf16:
                raise NotImplementedError("BF16 checkpoint snapshots cover the constant-density path only")
            gp.check_freq, gp.mute_radius_src, gp.mute_radius_rec = g.check_freq, g.mute_radius_src, g.mute_radius_rec
            gp.compute_misfit = int(g.compute_misfit)
        self._interp = int(getattr(matprop.interp_method, "code", 0))
        self._h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.sw_acoustic_vd_create(self.ctx.h, ctypes.byref(prm), self._interp, int(gradient),
                                                          ctypes.byref(gp), ctypes.byref(self._h)),
                       "sw_acoustic_vd_create")
        if runparams.compensated:
            self.ctx.check(self.ctx.lib.sw_acoustic_vd_set_precision(self._h, 1), "sw_acoustic_vd_set_precision")

    def __del__(self):
        try:
            if self._h:
                self.ctx.lib.sw_acoustic_vd_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass

    # -- checks (acou_models.jl:240-281) ----------------------------------------
    def check_matprop(self, matprop: VpRhoAcousticVDMaterialProperties):
        vp, rho = np.asarray(matprop.vp), np.asarray(matprop.rho)
        assert vp.ndim == rho.ndim == len(self.grid.size), \
            "Material property dimensionality must be the same as the wavesim!"
        assert vp.shape == rho.shape == self.grid.size, (
            f"Material property number of grid points must be the same as the wavesim! \n {vp.shape}, {rho.shape}, "
            f"{self.grid.size}")
        assert np.all(vp > 0), "Pressure velocity material property must be positive!"
        assert np.all(rho > 0), "Density material property must be positive!"
        courant = vd_courant_number(vp, self.dt, self.grid.spacing)
        log.info("Courant number: %s", courant)
        if self.runparams.erroronCFL:
            assert courant < 1, f"Courant number: {courant}"
        elif courant > 1:
            warnings.warn(f"CFL condition not satisfied! [{courant}]")

    def set_matprop(self, matprop: VpRhoAcousticVDMaterialProperties):
        """set_wavesim_matprop! -> update_matprop! + precompute_fact! (acou_models.jl:283-300)."""
        self.check_matprop(matprop)
        code = int(getattr(matprop.interp_method, "code", 0))
        if code != self._interp:
            raise ValueError("the interpolation method is fixed when the wavesim is built")
        self.matprop = VpRhoAcousticVDMaterialProperties(np.array(matprop.vp, copy=True), np.array(matprop.rho, copy=True),
                                                         matprop.interp_method)
        if self.runparams.compensated:  # the factors from the FP64 model
            vp64 = np.asfortranarray(matprop.vp, dtype=np.float64)
            rho64 = np.asfortranarray(matprop.rho, dtype=np.float64)
            self.ctx.check(self.ctx.lib.sw_acoustic_vd_set_material64(self._h, vp64.ctypes.data, rho64.ctypes.data),
                           "sw_acoustic_vd_set_material64")
            return
        vp32 = np.asfortranarray(matprop.vp, dtype=np.float32)
        rho32 = np.asfortranarray(matprop.rho, dtype=np.float32)
        self.ctx.check(self.ctx.lib.sw_acoustic_vd_set_material(self._h, vp32.ctypes.data, rho32.ctypes.data),
                       "sw_acoustic_vd_set_material")

    def possrcrec_scaletf(self, shot: ScalarShot):
        """acou_forward.jl:66-80: indices and tf * dt * vp(src)^2 rho(src) / prod(h)."""
        possrcs = nearest_grid_points(shot.srcs.positions, self.grid.spacing)
        posrecs = nearest_grid_points(shot.recs.positions, self.grid.spacing)
        return possrcs, posrecs, scale_srctf_vd(shot.srcs.tf, possrcs, self.matprop.vp, self.matprop.rho,
                                                self.grid.spacing, self.dt)

    def run_forward(self, shots):
        """Fills the seismograms; with RunParameters.snapevery returns, per shot, the
        reference's snapshot Dict {it: {"pcur": p, "vcur": [vx, vz]}} (acou_forward.jl:118-121)."""
        self.init_shots(shots)
        structs, keep = self._shot_structs(shots)
        snapevery = self.runparams.snapevery
        nx, nz = self.grid.size
        B = nx * nz + (nx - 1) * nz + nx * (nz - 1)
        if snapevery:
            bufs = [np.zeros((k[0].shape[0] // snapevery) * B, dtype=np.float32) for k in keep]
            ptrs = (ctypes.c_void_p * len(bufs))(*[b.ctypes.data for b in bufs])
            self.ctx.check(self.ctx.lib.sw_acoustic_vd_forward_snapshots(self._h, len(shots), structs, 0, snapevery,
                                                                         ptrs), "sw_acoustic_vd_forward_snapshots")
        else:
            self.ctx.check(self.ctx.lib.sw_acoustic_vd_forward(self._h, len(shots), structs, 0),
                           "sw_acoustic_vd_forward")
        for shot, (traces, _) in zip(shots, keep):
            shot.recs.seismograms[...] = traces
        if not snapevery:
            return None
        out = []
        for b in bufs:
            snaps = {}
            for q in range(len(b) // B):
                blk = b[q * B:(q + 1) * B]
                p = blk[:nx * nz].reshape((nx, nz), order="F").copy()
                vx = blk[nx * nz:nx * nz + (nx - 1) * nz].reshape((nx - 1, nz), order="F").copy()
                vz = blk[nx * nz + (nx - 1) * nz:].reshape((nx, nz - 1), order="F").copy()
                snaps[(q + 1) * snapevery] = {"pcur": p, "vcur": [vx, vz]}
            out.append(snaps)
        return out

    def run_gradient(self, shots, misfits):
        assert self.gradient, "The wavesim object was not built for gradient computations. (Was `gradient=true` specified?)"
        assert len(misfits) == len(shots)
        self.init_shots(shots)
        structs, keep = self._shot_structs(shots, misfits)
        g = {k: np.zeros(self.grid.size, dtype=np.float64, order="F") for k in ("vp", "rho")}
        misfit = np.zeros(1, dtype=np.float64)
        self.ctx.check(self.ctx.lib.sw_acoustic_vd_gradient(self._h, len(shots), structs, 0, g["vp"].ctypes.data,
                                                             g["rho"].ctypes.data, misfit.ctypes.data),
                       "sw_acoustic_vd_gradient")
        for shot, (traces, _) in zip(shots, keep):
            shot.recs.seismograms[...] = traces
        return g, float(misfit[0])

    def set_tuning(self, tz: int = 0, variant: int = 0):
        self.ctx.check(self.ctx.lib.sw_acoustic_vd_set_tuning(self._h, int(tz)), "sw_acoustic_vd_set_tuning")
