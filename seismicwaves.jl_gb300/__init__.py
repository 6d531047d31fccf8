"""seismicwaves.jl_gb300 -- GB300-native backend for SeismicWaves.jl's finite-difference hot path.

The compute path is libswgb300.so (hand-written sm_103a CUDA kernels behind
the C ABI of include/swgb300.h); this package is its host-side mirror of the
reference's Julia API (see ``api``).  The directory name contains a dot, so
import it through ``load_package()`` in ``__graft_entry__`` (or any
importlib loader) under the module name ``seismicwaves_gb300``.
"""
from . import _lib
from .api import (AcousticCDCPMLWaveSimulation, CCTSMisfit, CPMLBoundaryConditionParameters, GradParameters,
                  InputParametersAcoustic, L2Misfit, RunParameters, ScalarReceivers, ScalarShot, ScalarSources,
                  UniformFiniteDifferenceGrid, VpAcousticCDMaterialProperties, build_wavesim, courant_number, gaussderivstf,
                  gaussstf, nearest_grid_points, points_per_wavelength, rickerstf, scale_srctf,
                  swforward, swgradient, swmisfit)
from .elastic import (ArithmeticAverageInterpolation, ElasticIsoCPMLWaveSimulation, ElasticIsoMaterialProperties,
                      ExternalForceShot, ExternalForceSources, HarmonicAverageInterpolation, InputParametersElastic,
                      MomentTensor2D, MomentTensorShot, MomentTensorSources, VectorReceivers, spread_positions)
from .vd import AcousticVDStaggeredCPMLWaveSimulation, VpRhoAcousticVDMaterialProperties
from .rrules import GRADIENT_SIGN, misfit_function, rrule_swmisfit

__all__ = [
    "AcousticCDCPMLWaveSimulation", "CCTSMisfit", "CPMLBoundaryConditionParameters", "GradParameters", "InputParametersAcoustic",
    "L2Misfit", "RunParameters", "ScalarReceivers", "ScalarShot", "ScalarSources", "UniformFiniteDifferenceGrid",
    "VpAcousticCDMaterialProperties", "build_wavesim", "courant_number", "nearest_grid_points",
    "points_per_wavelength", "scale_srctf", "gaussderivstf", "gaussstf", "rickerstf", "swforward",
    "swgradient", "swmisfit", "_lib", "ArithmeticAverageInterpolation", "ElasticIsoCPMLWaveSimulation",
    "ElasticIsoMaterialProperties", "ExternalForceShot", "ExternalForceSources", "HarmonicAverageInterpolation",
    "InputParametersElastic", "MomentTensor2D", "MomentTensorShot", "MomentTensorSources", "VectorReceivers",
    "spread_positions", "AcousticVDStaggeredCPMLWaveSimulation", "VpRhoAcousticVDMaterialProperties",
    "GRADIENT_SIGN", "misfit_function", "rrule_swmisfit",
]
