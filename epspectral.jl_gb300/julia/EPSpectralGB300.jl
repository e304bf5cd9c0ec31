# EPSpectralGB300.jl -- the Julia side of the drop-in: `ccall` bindings of libepspectral_gb300.so
# and the two loop bodies EPSpectral.jl dispatches to when `backend isa GB300Backend`.
#
# It maps the `setup` NamedTuple of `_setup_scgd0` (src/scgd0.jl:173-183) and the ladder's
# additions (src/ladder.jl:153-157) onto `epsp_model` (include/epspectral_gb300.h), calls the
# library, and turns its status codes into the reference's errors (ArgumentError for EINVAL and
# ENOROOT_MU) and its convergence flags into the reference's warnings. Arrays are passed by pointer
# in their Julia (column-major) layout; index arrays are converted to 0-based Int32 once per call.
# A g2 of at most 1 GiB that the caller has pinned (`CUDA.pin(setup.g2)`, or `epsp_host_register`)
# is read in place by the plan set-ups' gather kernel; an unpinned one is gathered on the host.
# Not executed in this repository (no Julia toolchain here). To wire it, include this file from
# EPSpectral.jl and add a method of `_loop_scgd0` / `_loop_ladder` for `backend::GB300Backend` that
# calls `loop_scgd0` / `loop_ladder` below.
module EPSpectralGB300

const LIB = get(ENV, "EPSPECTRAL_GB300_LIB", joinpath(@__DIR__, "..", "epspectral_gb300", "libepspectral_gb300.so"))

const EPSP_OK, EPSP_EINVAL, EPSP_ENOMEM, EPSP_ENOROOT_MU = 0, 1, 2, 3
const PATHS = (direct_fp64 = Int32(0), gemm_fp64 = Int32(1), gemm_bf16 = Int32(2), gemm_tf32 = Int32(3))

"""The backend value `run_scgd0(...; backend = GB300Backend())` selects. With `keep_g2`, the
library keeps on the device the g2 the scGD0 set-up streams, and a ladder set-up of the same array
reads it there (a driver running `_loop_scgd0` and `_loop_ladder` on one setup; `run_scgd0_ladder`
extracts a new g2). The copy is freed after the next ladder set-up (epsp_ctx_keep_g2)."""
Base.@kwdef struct GB300Backend
    device::Int = 0
    path::Symbol = :gemm_bf16
    ladder_path::Union{Nothing, Symbol} = nothing  # the ladder's path when it differs (e.g. :gemm_tf32, ladder only)
    batch_rhs::Union{Nothing, Int} = nothing   # solve up to this many (T, Ω) pairs together (GMRES, :gemm_bf16)
    keep_g2::Bool = false
end

struct Grid
    origin::Float64
    unit::Float64
    offsets::Ptr{Int64}
    n::Int64
end

struct Model
    nm::Int64; ni::Int64; nf::Int64
    g2_dtype::Int32; reserved0::Int32; g2::Ptr{Cvoid}
    nq::Int64; omega_ph::Ptr{Float64}
    nk_i::Int64; nk_f::Int64; iq_kk::Ptr{Int32}
    iks_i::Ptr{Int32}; iks_f::Ptr{Int32}
    eps_i::Ptr{Float64}; w_i::Ptr{Float64}; eps_f::Ptr{Float64}; w_f::Ptr{Float64}
    f_to_i::Ptr{Int32}
    nmult::Int64; mult_ptr::Ptr{Int32}; mult_idx::Ptr{Int32}
    omegas::Grid; omegas_spectral::Grid
    W::Float64; nstates_base::Float64
    R::Ptr{Float64}; v::Ptr{Float64}
end

struct Options
    path::Int32; verbosity::Int32; gpu_tile::Int64; omega_acoustic::Float64
end

struct Occ
    nT::Int64; Tlist::Ptr{Float64}; nlist::Ptr{Float64}; nelec::Float64; spin_degeneracy::Float64
    type::Int32; reserved0::Int32
end

mutable struct History
    err::Ptr{Float64}; mu::Ptr{Float64}; min_spectral_weight::Ptr{Float64}; wall::Ptr{Float64}
    iter_frozen::Ptr{Int32}; niter::Int32; reserved0::Int32
end

function check(ctx, status)
    status == EPSP_OK && return nothing
    msg = unsafe_string(ccall((:epsp_last_error, LIB), Cstring, (Ptr{Cvoid},), ctx))
    status in (EPSP_EINVAL, EPSP_ENOROOT_MU) && throw(ArgumentError(msg))
    error("libepspectral_gb300: status $status: $msg")
end

# One library context per device for the process (its stream, its page-locked staging and the g2
# it keeps live across calls), created on first use and destroyed at exit. The library's calls on
# one context are not concurrent: LOCK serialises the loops.
const CONTEXTS = Dict{Int, Ptr{Cvoid}}()
const LOCK = ReentrantLock()

function __init__()
    atexit() do
        for ctx in values(CONTEXTS)
            ccall((:epsp_destroy, LIB), Cvoid, (Ptr{Cvoid},), ctx)
        end
        empty!(CONTEXTS)
    end
end

function context(backend::GB300Backend)
    get!(CONTEXTS, backend.device) do
        ref = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:epsp_create, LIB), Cint, (Ref{Ptr{Cvoid}}, Int32), ref, backend.device)
        st == EPSP_OK || error("epsp_create failed with status $st")
        ref[]
    end
end

"""
    host_register(backend, A) / host_unregister(backend, A)

Page-lock the memory of the dense array `A` for the library (epsp_host_register): plan set-ups
then read a g2 of at most 1 GiB there in place. `CUDA.pin(A)` does the same. Unregister before
`A` is freed.
"""
function host_register(backend::GB300Backend, A::Array)
    lock(LOCK) do
        ctx = context(backend)
        check(ctx, ccall((:epsp_host_register, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, UInt64), ctx, pointer(A),
            sizeof(A)))
    end
end
function host_unregister(backend::GB300Backend, A::Array)
    lock(LOCK) do
        ctx = context(backend)
        check(ctx, ccall((:epsp_host_unregister, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx, pointer(A)))
    end
end

dtype_tag(::Type{Float64}) = Int32(0)
dtype_tag(::Type{Float32}) = Int32(1)

# The arrays the model struct points at; kept alive by the caller with GC.@preserve.
function model_arrays(setup, R, v)
    (; g2, ωph, iq_kk, iks_i, iks_f, ε_i, w_i, ε_f, w_f, f_to_i, W, nstates_base, multiplets, ωs, ωs_spectral) = setup
    zb(x) = Int32.(Array(x) .- 1)   # 1-based Julia indices -> 0-based Int32
    # g2 is passed as the caller's own array when it is dense, so that its address is the same in
    # both set-ups of a run (the kept copy) and a pinned g2 is the memory the library reads
    g2 = g2 isa Array ? g2 : Array(g2)
    mult_ptr = Int32[0; cumsum(length.(multiplets))]
    mult_idx = isempty(multiplets) ? Int32[0] : Int32.(reduce(vcat, multiplets) .- 1)
    (; g2, ωph = Array(ωph), iq_kk = zb(iq_kk), iks_i = zb(iks_i), iks_f = zb(iks_f),
       ε_i = Array(ε_i), w_i = Array(w_i), ε_f = Array(ε_f), w_f = Array(w_f), f_to_i = zb(f_to_i),
       W, nstates_base, mult_ptr, mult_idx, offsets = collect(Int64, ωs.offsets), ωs,
       offsets_sp = collect(Int64, ωs_spectral.offsets), ωs_spectral,
       R = R === nothing ? nothing : Array{Float64}(R), v = v === nothing ? nothing : Array{Float64}(v))
end

function model_struct(a)
    nm, ni, nf = size(a.g2)
    Model(nm, ni, nf, dtype_tag(eltype(a.g2)), 0, pointer(a.g2), size(a.ωph, 2), pointer(a.ωph),
        size(a.iq_kk, 1), size(a.iq_kk, 2), pointer(a.iq_kk), pointer(a.iks_i), pointer(a.iks_f),
        pointer(a.ε_i), pointer(a.w_i), pointer(a.ε_f), pointer(a.w_f), pointer(a.f_to_i),
        length(a.mult_ptr) - 1, pointer(a.mult_ptr), pointer(a.mult_idx),
        Grid(a.ωs.ω_origin, a.ωs.dω_unit, pointer(a.offsets), length(a.offsets)),
        Grid(a.ωs_spectral.ω_origin, a.ωs_spectral.dω_unit, pointer(a.offsets_sp), length(a.offsets_sp)),
        a.W, a.nstates_base,
        a.R === nothing ? Ptr{Float64}(C_NULL) : pointer(a.R), a.v === nothing ? Ptr{Float64}(C_NULL) : pointer(a.v))
end

"""
    loop_scgd0(setup, occ; η_min, η_init, maxiter, tol, backend::GB300Backend, gpu_tile, Σ_init,
               fix_μ, ω_acoustic, verbosity)

The body of EPSpectral's `_loop_scgd0` (src/scgd0.jl:189-346) on the GB300 library, with the
same arguments and the same return value `(; Σ, μ, converged, history)`.
"""
function loop_scgd0(setup, occ; η_min, η_init, maxiter, tol, backend::GB300Backend, gpu_tile, Σ_init, fix_μ,
        ω_acoustic, verbosity)
    lock(LOCK) do
        ctx = context(backend)
        a = model_arrays(setup, nothing, nothing)
        nω, ni, nT = length(setup.ωs), size(setup.g2, 2), length(occ.Tlist)
        Tlist, nlist = collect(Float64, occ.Tlist), collect(Float64, occ.nlist)
        μ_start = collect(Float64, setup.μ_start)
        ηm = collect(Float64, η_min)
        Σ_in = Σ_init === nothing ? nothing : Array{ComplexF64}(Σ_init)
        Σ = Array{ComplexF64}(undef, nω, ni, nT)
        μ = zeros(nT); conv = zeros(UInt8, nT)
        err, hμ, hA = (fill(NaN, nT, maxiter) for _ in 1:3)
        wall = zeros(maxiter); frozen = zeros(Int32, nT)
        GC.@preserve a Tlist nlist μ_start ηm Σ_in Σ μ conv err hμ hA wall frozen begin
            m = Ref(model_struct(a))
            opts = Ref(Options(getfield(PATHS, backend.path), verbosity, gpu_tile === nothing ? 0 : gpu_tile, ω_acoustic))
            plan = Ref{Ptr{Cvoid}}(C_NULL)
            backend.keep_g2 && check(ctx, ccall((:epsp_ctx_keep_g2, LIB), Cint, (Ptr{Cvoid}, Int32), ctx, 1))
            check(ctx, ccall((:epsp_scgd0_setup, LIB), Cint, (Ptr{Cvoid}, Ref{Model}, Ref{Options}, Ref{Ptr{Cvoid}}),
                ctx, m, opts, plan))
            try
                o = Ref(Occ(nT, pointer(Tlist), pointer(nlist), occ.nelec, occ.spin_degeneracy,
                    occ.type === :Semiconductor ? 1 : 0, 0))
                h = Ref(History(pointer(err), pointer(hμ), pointer(hA), pointer(wall), pointer(frozen), 0, 0))
                check(ctx, ccall((:epsp_scgd0_run, LIB), Cint,
                    (Ptr{Cvoid}, Ref{Occ}, Ptr{Float64}, Float64, Int32, Float64, Int32, Ptr{Float64}, Ptr{ComplexF64},
                     Ptr{ComplexF64}, Ptr{Float64}, Ptr{UInt8}, Ref{History}),
                    plan[], o, ηm, η_init, maxiter, tol, fix_μ, μ_start,
                    Σ_in === nothing ? Ptr{ComplexF64}(C_NULL) : pointer(Σ_in), Σ, μ, conv, h))
                n = h[].niter
                any(iszero, conv) && maxiter > 1 && @warn "scGD0 not converged after maxiter = $maxiter iterations at T = $(occ.Tlist[iszero.(conv)])"
                history = (; err = err[:, 1:n], μ = hμ[:, 1:n], min_spectral_weight = hA[:, 1:n], wall = wall[1:n],
                           iter_frozen = Int.(frozen))
                return (; Σ, μ, converged = Vector{Bool}(conv .!= 0), history)
            finally
                ccall((:epsp_scgd0_plan_destroy, LIB), Cvoid, (Ptr{Cvoid},), plan[])
            end
        end
    end
end

"""
    loop_ladder(ladder, Σ, μ, Tlist, Ωs; solver, rtol, maxiter, store_vertex, backend::GB300Backend,
                gpu_tile, ω_acoustic, verbosity)

The body of EPSpectral's `_loop_ladder` (src/ladder.jl:303-379) on the GB300 library. `ladder` is
the output of `_setup_ladder`, whose rotations `R` and velocities `v` are passed as dense arrays.
"""
function loop_ladder(ladder, Σ, μ, Tlist, Ωs; solver, rtol, maxiter, store_vertex, backend::GB300Backend,
        gpu_tile, ω_acoustic, verbosity)
    lock(LOCK) do
        ctx = context(backend)
        a = model_arrays(ladder, Array(ladder.R), Array(ladder.v))
        nω, ni = length(ladder.ωs), size(ladder.g2, 2)
        nT, nΩ = length(Tlist), length(Ωs)
        Σh, μh = Array{ComplexF64}(Σ), collect(Float64, μ)
        Th, Ωh = collect(Float64, Tlist), collect(Float64, Ωs)
        σb, σl = zeros(3, 3, nΩ, nT), zeros(3, 3, nΩ, nT)
        conv, niter = zeros(UInt8, nΩ, nT), zeros(Int32, nΩ, nT)
        J = store_vertex ? zeros(ComplexF64, nω, 4, 3, 2, ni, nΩ, nT) : nothing
        GC.@preserve a Σh μh Th Ωh σb σl conv niter J begin
            m = Ref(model_struct(a))
            lpath = backend.ladder_path === nothing ? backend.path : backend.ladder_path
            opts = Ref(Options(getfield(PATHS, lpath), verbosity, gpu_tile === nothing ? 0 : gpu_tile, ω_acoustic))
            plan = Ref{Ptr{Cvoid}}(C_NULL)
            try
                check(ctx, ccall((:epsp_ladder_setup, LIB), Cint,
                    (Ptr{Cvoid}, Ref{Model}, Ref{Options}, Ref{Ptr{Cvoid}}), ctx, m, opts, plan))
            finally  # the ladder's set-up was the kept g2's last reader
                backend.keep_g2 && ccall((:epsp_ctx_keep_g2, LIB), Cint, (Ptr{Cvoid}, Int32), ctx, 0)
            end
            try
                Jp = J === nothing ? Ptr{ComplexF64}(C_NULL) : pointer(J)
                if backend.batch_rhs !== nothing && solver === :gmres
                    # every (T, Ω) pair from x0 = 0, up to batch_rhs of them per operator application
                    check(ctx, ccall((:epsp_ladder_run_batched, LIB), Cint,
                        (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Float64,
                         Int32, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{UInt8}, Ptr{Int32}, Ptr{Cvoid}, Ptr{ComplexF64}),
                        plan[], Σh, μh, Th, nT, Ωh, nΩ, rtol, maxiter, backend.batch_rhs, σb, σl, conv, niter,
                        C_NULL, Jp))
                else
                    check(ctx, ccall((:epsp_ladder_run, LIB), Cint,
                        (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Int32, Float64,
                         Int32, Ptr{Float64}, Ptr{Float64}, Ptr{UInt8}, Ptr{Int32}, Ptr{Cvoid}, Ptr{ComplexF64}),
                        plan[], Σh, μh, Th, nT, Ωh, nΩ, solver === :gmres ? 0 : 1, rtol, maxiter, σb, σl, conv, niter,
                        C_NULL, Jp))
                end
            finally
                ccall((:epsp_ladder_plan_destroy, LIB), Cvoid, (Ptr{Cvoid},), plan[])
            end
        end
        converged = conv .!= 0
        all(converged) || @warn "ladder not converged (rtol = $rtol, maxiter = $maxiter)"
        history = fill((; norms = Float64[], σ_iter = Matrix{Float64}[]), nΩ, nT)
        return (; σ_bubble = σb, σ_ladder = σl, converged, niter = Int.(niter), history, J)
    end
end

end # module
