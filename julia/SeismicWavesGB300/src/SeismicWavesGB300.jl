"""
    SeismicWavesGB300

GB300 backend of SeismicWaves.jl: `using SeismicWaves, SeismicWavesGB300`
and `RunParameters(parall = :GB300)` route `swforward!`, `swmisfit!` and
`swgradient!` of the acoustic constant-density (2D, 3D), variable-density (2D)
and isotropic elastic (2D) C-PML simulations to `libswgb300.so`, with all
shots of a call batched on one GPU.  SeismicWaves.jl itself is unchanged:
select_backend (src/models/backend_selection.jl:2-40) gains a `Val{:GB300}`
method, as the package's own CUDA extension does
(ext/SeismicWaves_CUDABackendExt.jl:13-25), and the shot loops dispatch on the
resulting wavesim type (see backend.jl).
"""
module SeismicWavesGB300

using LinearAlgebra: isdiag, diag
using SeismicWaves
using SeismicWaves: CPMLBoundaryCondition, LocalGrid, AcousticCDCPMLWaveSimulation,
                    AcousticVDStaggeredCPMLWaveSimulation, ElasticIsoCPMLWaveSimulation, possrcrec_scaletf,
                    init_shot!, check_sim_consistency, set_wavesim_matprop!, snapenabled

export GB300Array, set_library!, set_device!, release!

include("abi.jl")
include("backend.jl")
include("acoustic.jl")
include("elastic.jl")

end # module
