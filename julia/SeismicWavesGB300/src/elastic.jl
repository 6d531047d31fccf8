# run_swforward! / run_swgradient! for ElasticIsoCPMLWaveSimulation built with
# parall = :GB300 (moment-tensor and external-force shots, vector receivers).
# The source / receiver point tables are the reference's own possrcrec_scaletf
# output (spread_positions with sincinterp, one nearest point otherwise,
# src/models/elastic/ela_models.jl:6-90), packed as CSR per item.

function elastic_handle(model::GB300Elastic)
    handle(model) do ctx
        nx, nz = model.grid.size
        hx, hz = model.grid.spacing
        cp = model.cpmlparams
        harmonic(m) = m isa SeismicWaves.HarmonicAverageInterpolation ? Int32(1) : Int32(0)
        p = SwElasticParams((Int32(nx), Int32(nz)), (Float64(hx), Float64(hz)), Float64(model.dt), Int32(cp.halo),
                            Float64(cp.rcoef), Int32(cp.freeboundtop), harmonic(model.matprop.interp_method_ρ),
                            harmonic(model.matprop.interp_method_μ))
        g = grad_params(model)
        es = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:sw_elastic_create, libsw[]), Cint,
                    (Ptr{Cvoid}, Ref{SwElasticParams}, Int32, Ref{SwGradParams}, Ref{Ptr{Cvoid}}),
                    ctx, p, Int32(isgradsim(model)), g, es), ctx, "sw_elastic_create")
        GB300Handle(ctx, es[], :sw_elastic_destroy)
    end
end

function set_material!(h::GB300Handle, model::GB300Elastic)
    mp = model.matprop
    lam, mu, rho = Float32.(mp.λ), Float32.(mp.μ), Float32.(mp.ρ)
    check(ccall((:sw_elastic_set_material, libsw[]), Cint, (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}),
                h.sim, lam, mu, rho), h.ctx, "sw_elastic_set_material")
end

# (idx_i, coeffs_i) per item, as spread_positions returns them -> CSR
# (offsets (n+1), ij (2, npoints), coef (npoints))
function csr(idxs, coeffs)
    off = Int32[0; cumsum(length.(coeffs))]
    ij = Int32.(vcat([permutedims(m) for m in idxs]...)')[:]
    return off, ij, Float32.(vcat(coeffs...))
end

struct ElasticShotBuffers
    tabs::NTuple{4, Tuple{Vector{Int32}, Vector{Int32}, Vector{Float32}}}  # src 1, src 2, rec ux, rec uz
    tf::Matrix{Float32}
    momtens::Matrix{Float32}
    tr::Array{Float32, 3}
    cp::Vector{Float32}
    obs::Union{Nothing, Array{Float32, 3}}
    icd::Union{Nothing, Vector{Float32}}
    icf::Union{Nothing, Matrix{Float32}}
    win::Vector{Int32}
    sp::Matrix{Float64}
    rp::Matrix{Float64}
    kind::Int32
    mkind::Int32
    mdt::Float64
end

function elastic_shot_buffers(model, shot, misfit)
    init_shot!(model, shot)
    s1ij, s1c, s2ij, s2c, ruxij, ruxc, ruzij, ruzc, scal = possrcrec_scaletf(model, shot; sincinterp=model.sincinterp)
    tabs = (csr(s1ij, s1c), csr(s2ij, s2c), csr(ruxij, ruxc), csr(ruzij, ruzc))
    kind = shot isa SeismicWaves.MomentTensorShot ? Int32(0) : Int32(1)
    momtens = kind == 0 ? Float32.(hcat([[m.Mxx, m.Mzz, m.Mxz] for m in shot.srcs.momtens]...)) : zeros(Float32, 3, 0)
    obs, icd, icf, win, mkind, mdt = nothing, nothing, nothing, Int32[], Int32(0), 0.0
    if misfit !== nothing
        icd, icf, win, mkind, mdt = misfit_fields(misfit)
        obs = Float32.(misfit.observed)
    end
    tr = zeros(Float32, size(shot.recs.seismograms))
    return ElasticShotBuffers(tabs, Float32.(scal), momtens, tr, cpml_block(model), obs, icd, icf, win,
                              Float64.(shot.srcs.positions), Float64.(shot.recs.positions), kind, mkind, mdt)
end

pt(t) = SwPointTable(pointer(t[1]), pointer(t[2]), pointer(t[3]))

sw_struct(b::ElasticShotBuffers) =
    SwElasticShot(Int32(size(b.tr, 1)), b.kind, Int32(size(b.sp, 1)), pointer(b.tf),
                  isempty(b.momtens) ? Ptr{Float32}(C_NULL) : pointer(b.momtens), (pt(b.tabs[1]), pt(b.tabs[2])),
                  Int32(size(b.rp, 1)), (pt(b.tabs[3]), pt(b.tabs[4])), pointer(b.tr), pointer(b.cp), optptr(b.obs),
                  optptr(b.icd), Int32(length(b.win) ÷ 2), isempty(b.win) ? Ptr{Int32}(C_NULL) : pointer(b.win),
                  pointer(b.sp), pointer(b.rp), optptr(b.icf), b.mkind, b.mdt)

function save_snapshots!(model::GB300Elastic{T}, buf::Vector{Float32}, nt::Int) where {T}
    nx, nz = model.grid.size
    sizes = ((nx - 1, nz), (nx, nz - 1), (nx, nz), (nx, nz), (nx - 1, nz - 1))
    B = sum(prod, sizes)
    k = 0
    for it in 1:nt
        it % model.snapshotter.snapevery == 0 || continue
        o = k * B
        parts = Array{T, 2}[]
        for s in sizes
            push!(parts, reshape(T.(buf[(o + 1):(o + prod(s))]), s))
            o += prod(s)
        end
        SeismicWaves.savesnapshot!(model.snapshotter, "ucur" => SeismicWaves.MultiVariableField(parts[1:2]), it)
        SeismicWaves.savesnapshot!(model.snapshotter, "σ" => SeismicWaves.MultiVariableField(parts[3:5]), it)
        k += 1
    end
end

function SeismicWaves.run_swforward!(model::GB300Elastic, matprop::SeismicWaves.MaterialProperties{T, N},
                                     shots::Vector{<:SeismicWaves.Shot{T}}) where {T, N}
    check_sim_consistency(model, matprop, shots)
    set_wavesim_matprop!(model, matprop)
    h = elastic_handle(model)
    set_material!(h, model)
    bufs = [elastic_shot_buffers(model, shot, nothing) for shot in shots]
    structs = [sw_struct(b) for b in bufs]
    if snapenabled(model)
        every = model.snapshotter.snapevery
        nx, nz = model.grid.size
        B = (nx - 1) * nz + nx * (nz - 1) + 2 * nx * nz + (nx - 1) * (nz - 1)
        snaps = [zeros(Float32, B * (size(b.tr, 1) ÷ every)) for b in bufs]
        ptrs = [pointer(s) for s in snaps]
        GC.@preserve bufs snaps ptrs structs check(ccall((:sw_elastic_forward_snapshots, libsw[]), Cint,
                                                         (Ptr{Cvoid}, Int32, Ptr{SwElasticShot}, Int32, Int32,
                                                          Ptr{Ptr{Float32}}),
                                                         h.sim, length(structs), structs, 0, every, ptrs),
                                                   h.ctx, "sw_elastic_forward_snapshots")
        out = []
        for (shot, b, s) in zip(shots, bufs, snaps)
            shot.recs.seismograms .= b.tr
            save_snapshots!(model, s, size(b.tr, 1))
            push!(out, deepcopy(model.snapshotter.snapshots))
        end
        return out
    end
    GC.@preserve bufs structs check(ccall((:sw_elastic_forward, libsw[]), Cint,
                                          (Ptr{Cvoid}, Int32, Ptr{SwElasticShot}, Int32),
                                          h.sim, length(structs), structs, 0), h.ctx, "sw_elastic_forward")
    for (shot, b) in zip(shots, bufs)
        shot.recs.seismograms .= b.tr
    end
    return nothing
end

function SeismicWaves.run_swgradient!(model::GB300Elastic, matprop::SeismicWaves.MaterialProperties{T, N},
                                      shots::Vector{<:SeismicWaves.Shot{T}},
                                      misfit::Vector{<:SeismicWaves.AbstractMisfit{T}}) where {T, N}
    @assert model.checkpointer !== nothing "The wavesim object was not built for gradient computations. (Was `gradient=true` specified?)"
    check_sim_consistency(model, matprop, shots)
    set_wavesim_matprop!(model, matprop)
    h = elastic_handle(model)
    set_material!(h, model)
    bufs = [elastic_shot_buffers(model, shot, m) for (shot, m) in zip(shots, misfit)]
    structs = [sw_struct(b) for b in bufs]
    grho = zeros(Float64, model.grid.size)
    glam = zeros(Float64, model.grid.size)
    gmu = zeros(Float64, model.grid.size)
    msf = Ref(0.0)
    GC.@preserve bufs structs check(ccall((:sw_elastic_gradient, libsw[]), Cint,
                                          (Ptr{Cvoid}, Int32, Ptr{SwElasticShot}, Int32, Ptr{Float64}, Ptr{Float64},
                                           Ptr{Float64}, Ref{Float64}),
                                          h.sim, length(structs), structs, 0, grho, glam, gmu, msf),
                                    h.ctx, "sw_elastic_gradient")
    for (shot, b) in zip(shots, bufs)
        shot.recs.seismograms .= b.tr
    end
    g = Dict("rho" => T.(grho), "lambda" => T.(glam), "mu" => T.(gmu))
    return model.gradparams.compute_misfit ? (g, T(msf[])) : g
end
