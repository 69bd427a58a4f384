# XcoreGPU.jl -- Julia binding of libxcore_gb300.so (include/xcore_gb300.h).
#
# Drop-in for the per-timestep functions of xcore.jl: the functions below keep
# the reference's names and keyword arguments and forward to the GB300 library
# through ccall.  The state lives on the GPU inside a context; `upload!` /
# `download!` move a reference FluidState / PhaseState / NoiseState field by
# field (same names, same column-major sizes, Float64, Bool for hasx/hasm).
#
# Usage (after `initialize!` on the host, or with `initialize_gpu!`):
#     gpu = XcoreGPU.Context(par, grid, scales)
#     XcoreGPU.upload!(gpu, phase, fluid, ns)
#     for step in 1:nsteps
#         XcoreGPU.step!(gpu, step, dt, randn(rng, Nz, Nx), randn(rng, Nz, Nx))
#     end
#     XcoreGPU.download!(gpu, phase, fluid, ns)
module XcoreGPU

import xcore

const LIB = joinpath(@__DIR__, "..", "_build", "libxcore_gb300.so")

const SCHEMES = Dict(:centr => 0, :upwd1 => 1, :quick => 2, :fromm => 3, :weno3 => 4, :weno5 => 5, :tvdim => 6)
const BCS = Dict(:periodic => 0, :closed => 1)
const TINTS = Dict(:be1im => 0, :bd2im => 1, :cn2si => 2, :bd2si => 3)

# mirrors xc_params (field order and types must match the C struct)
struct XcParams
    Nz::Cint; Nx::Cint; h::Cdouble; D::Cdouble
    rhom0::Cdouble; rhox0::Cdouble; d0::Cdouble; g0::Cdouble; etam0::Cdouble; etax0::Cdouble
    AA::NTuple{4,Cdouble}; BB::NTuple{4,Cdouble}; CC::NTuple{4,Cdouble}
    Xi::Cdouble; Ptop::Cdouble; alpha::Cdouble; gamma::Cdouble; CFL::Cdouble; dtmax::Cdouble
    etacntr::Cdouble; open_sgr::Cint
    L0::Cdouble; l0::Cdouble; L0h::Cdouble; l0h::Cdouble; D0::Cdouble; txi0::Cdouble
    G0::Cdouble; bnd_w::Cdouble; dt0::Cdouble
    ADVN::Cint; TINT::Cint; xBC::Cint; zBC::Cint
    sds::Cint; top_cnv::Cint; bot_cnv::Cint; open_cnv::Cint
    weno_weights::Cint
end

struct SolverOpts
    kind::Cint; rtol::Cdouble; maxit::Cint; restart::Cint; inner_rtol::Cdouble; inner_maxit::Cint
    smooth_sweeps::Cint; omega_velocity::Cdouble; schur_mass::Cdouble; schur_full_diagonal::Cint
    coarse_cells::Cint; coarse_sweeps::Cint; small_cells::Cint; pressure_sweeps::Cint; inner_gs_passes::Cint
    serial_launch::Cint; coarse_viscosity_mean::Cint; tiled_sweep::Cint; post_sweeps::Cint; outer_solver::Cint
    fused_pressure_cells::Cint; stage_small_levels::Cint; jacobi_coarse::Cint; row_block_sweep::Cint; learned::Cint
    device_givens::Cint; cluster_cells::Cint
end
SolverOpts(kind, rtol, maxit, restart, inner_rtol, inner_maxit) =
    SolverOpts(kind, rtol, maxit, restart, inner_rtol, inner_maxit, 0, 0.0, 0.0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0)

struct SolverStats
    iterations::Cint; refinements::Cint; rel_residual::Cdouble; converged::Cint; seconds::Cdouble
    learned_fallbacks::Cint; device_givens_steps::Cint
end

const MAX_SWEEPS = 64
# mirrors xc_step_stats
struct StepStats
    resnorm::NTuple{64,Cdouble}; resnorm0::Cdouble; sweeps::Cint; solver_iterations::Cint
    solver_rel_residual::Cdouble; dt_next::Cdouble; unconverged_solves::Cint; picard_converged::Cint
end
StepStats() = StepStats(ntuple(_ -> 0.0, MAX_SWEEPS), 0.0, 0, 0, 0.0, 0.0, 0, 0)

mutable struct Context
    h::Ptr{Cvoid}
    Nz::Int
    Nx::Int
end

check(st) = st == 0 ? nothing :
    error("xcore_gb300 status $st: " * unsafe_string(ccall((:xc_last_error, LIB), Cstring, ())))

row(m) = (Cdouble(m[1, 1]), Cdouble(m[1, 2]), Cdouble(m[2, 1]), Cdouble(m[2, 2]))

function Context(par, grid, scales; xBC = :periodic, zBC = :closed, sds = -1, top_cnv = 1, bot_cnv = 1,
                 open_cnv = false, weno_weights = 0)
    p = XcParams(grid.Nz, grid.Nx, grid.h, par.D, par.rhom0, par.rhox0, par.d0, par.g0, par.etam0, par.etax0,
                 row(par.AA), row(par.BB), row(par.CC), par.Xi, par.Ptop, par.alpha, par.gamma, par.CFL,
                 par.dtmax, par.etacntr, par.open_sgr,
                 scales.L0, scales.l0, scales.L0h, scales.l0h, scales.D0, scales.txi0, scales.G0, scales.bnd_w,
                 scales.dt0, SCHEMES[par.ADVN], TINTS[par.TINT], BCS[xBC], BCS[zBC], sds, top_cnv, bot_cnv,
                 open_cnv, weno_weights)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:xc_ctx_create, LIB), Cint, (Ref{XcParams}, Ref{Ptr{Cvoid}}), p, h))
    ctx = Context(h[], grid.Nz, grid.Nx)
    finalizer(c -> ccall((:xc_ctx_destroy, LIB), Cint, (Ptr{Cvoid},), c.h), ctx)
    return ctx
end

fieldid(name::Symbol) = ccall((:xc_field_id, LIB), Cint, (Cstring,), String(name))

function upload!(ctx::Context, name::Symbol, a::AbstractMatrix)
    id = fieldid(name)
    id < 0 && return
    host = eltype(a) == Bool ? Matrix{UInt8}(a) : Matrix{Float64}(a)
    check(ccall((:xc_field_upload, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}), ctx.h, id, host))
end

function download!(ctx::Context, name::Symbol, a::AbstractMatrix)
    id = fieldid(name)
    id < 0 && return
    if eltype(a) == Bool
        tmp = Matrix{UInt8}(undef, size(a))
        check(ccall((:xc_field_download, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}), ctx.h, id, tmp))
        a .= tmp .!= 0
    else
        check(ccall((:xc_field_download, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}), ctx.h, id, a))
    end
    return a
end

# every matrix field of the reference structs that the library also holds
function foreach_field(f, structs...)
    for s in structs, name in fieldnames(typeof(s))
        v = getfield(s, name)
        v isa AbstractMatrix && fieldid(name) >= 0 && f(name, v)
    end
end

upload!(ctx::Context, structs...) = foreach_field((n, v) -> upload!(ctx, n, v), structs...)
download!(ctx::Context, structs...) = foreach_field((n, v) -> download!(ctx, n, v), structs...)

# ---- checkpoints (src/restart.jl:53-127) -------------------------------------------
# The reference's own JLD2 writer and reader, with the device state moved through
# download!/upload! (every array of FluidState, PhaseState and the NoiseState
# fields the library holds).  The noise RNG never leaves Julia -- the library takes
# each step's white-noise draws as inputs -- so ns.rng is saved and restored by the
# reference code unchanged, and a GPU run resumes from a CPU checkpoint or the
# other way round.
function save_checkpoint(ctx::Context, path, phase, fluid, ns, hst; time, dt, step)
    download!(ctx, phase, fluid, ns)
    xcore.save_checkpoint(path, phase, fluid, ns, hst; time = time, dt = dt, step = step)
end

function load_checkpoint!(ctx::Context, path, phase, fluid, ns, hst)
    r = xcore.load_checkpoint!(path, phase, fluid, ns, hst)
    upload!(ctx, phase, fluid, ns)
    return r
end

coefs(a1, a2, a3, b1, b2, b3) = Cdouble[a1, a2, a3, b1, b2, b3]

# ---- the reference's functions ------------------------------------------------------
store_previous!(ctx::Context) = check(ccall((:xc_store_previous, LIB), Cint, (Ptr{Cvoid},), ctx.h))
store_noise!(ctx::Context) = check(ccall((:xc_store_noise, LIB), Cint, (Ptr{Cvoid},), ctx.h))
snapshot!(ctx::Context) = check(ccall((:xc_snapshot, LIB), Cint, (Ptr{Cvoid},), ctx.h))

function phsevo!(ctx::Context; ADVN::Symbol = :weno5, a1, a2, a3, b1, b2, b3, dt, alpha)
    check(ccall((:xc_phsevo, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cdouble, Cdouble),
                ctx.h, SCHEMES[ADVN], coefs(a1, a2, a3, b1, b2, b3), dt, alpha))
end

function fluidmech!(ctx::Context; dt, a1 = 1.0, a2 = 1.0, a3 = 0.0, b1 = 1.0, b2 = 0.0, b3 = 0.0,
                    solver::Symbol = :fgmres64, rtol = 1e-10, maxit = 500)
    o = SolverOpts(solver === :mixed ? 1 : 0, rtol, maxit, 30, 1e-3, 40)
    s = Ref{SolverStats}()
    check(ccall((:xc_fluidmech, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cdouble, Ref{SolverOpts}, Ref{SolverStats}),
                ctx.h, coefs(a1, a2, a3, b1, b2, b3), dt, o, s))
    return s[]
end

function noise!(ctx::Context, dt; first_iter::Bool = true, re = nothing, rs = nothing)
    # ccall keeps the converted arrays alive for the duration of the call
    hre = re === nothing ? Ptr{Cdouble}(C_NULL) : Matrix{Float64}(re)
    hrs = rs === nothing ? Ptr{Cdouble}(C_NULL) : Matrix{Float64}(rs)
    check(ccall((:xc_noise, LIB), Cint, (Ptr{Cvoid}, Cdouble, Cint, Ptr{Cdouble}, Ptr{Cdouble}),
                ctx.h, dt, first_iter, hre, hrs))
end

update_phase_velocities!(ctx::Context) =
    check(ccall((:xc_update_phase_velocities, LIB), Cint, (Ptr{Cvoid},), ctx.h))
update!(ctx::Context) = check(ccall((:xc_update, LIB), Cint, (Ptr{Cvoid},), ctx.h))

function update_dt(ctx::Context, dt_prev)
    out = Ref{Cdouble}()
    check(ccall((:xc_update_dt, LIB), Cint, (Ptr{Cvoid}, Cdouble, Ref{Cdouble}), ctx.h, dt_prev, out))
    return out[]
end

function compute_resnorm(ctx::Context, dt)
    out = zeros(Cdouble, 3)
    check(ccall((:xc_resnorm, LIB), Cint, (Ptr{Cvoid}, Cdouble, Ptr{Cdouble}), ctx.h, dt, out))
    return (out[1], out[2], out[3])
end

# one outer step of run! with `sweeps` Picard sweeps; returns the next dt
# ---- values record_history! pushes (src/history.jl:121-145, 183-222) ---------------
# {sumB, sumM, sumX, sumGx, top_aX, bot_aX, top_aM, bot_aM, top_dX, bot_dX, top_dM, bot_dM}
function conservation_sums(ctx::Context)
    out = Vector{Cdouble}(undef, 12)
    check(ccall((:xc_conservation_sums, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), ctx.h, out))
    return out
end

const HISTORY_KEYS = vcat(["x_min", "x_mean", "x_max", "x_std"],
                          ["$(f)_$(s)" for f in ("V", "vx", "vm", "xie", "xix", "xis") for s in ("min", "rms", "max")],
                          ["$(f)_$(s)" for f in ("Ra", "Rc", "ReD", "Red", "ks", "ke", "kx", "eta", "etamix", "etae",
                                                 "etas", "etat") for s in ("min", "gm", "max")])

function history_stats(ctx::Context)
    out = Vector{Cdouble}(undef, 58)
    check(ccall((:xc_history_stats, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), ctx.h, out))
    return Dict(zip(HISTORY_KEYS, out))
end

# The statistics print_step! prints beyond record_history!'s (src/diagnose.jl:92-182),
# on the raw fields (divide by the scales as print_step! does before printing)
const PRINT_KEYS = vcat(["m_min", "m_mean", "m_max"],
                        ["$(f)_$(s)" for f in ("rho", "V", "vx", "vm", "xie", "xix", "xis") for s in ("min", "gm", "max")])

function print_step_stats(ctx::Context)
    out = Vector{Cdouble}(undef, 24)
    check(ccall((:xc_print_step_stats, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), ctx.h, out))
    return Dict(zip(PRINT_KEYS, out))
end

# the measured optimum of the 1024^2 time step: FP32 inner solves to a 5e-2
# reduction in at most 30 iterations, one pressure-multigrid sweep; at most 400
# FP32 iterations per mixed solve, 3000 per plain FP64 solve
step_solver_opts(solver::Symbol, rtol; learned = 0) =
    SolverOpts(solver === :mixed ? 1 : 0, rtol, solver === :mixed ? 400 : 3000, 30, 5e-2, 30,
               0, 0.0, 0.0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, learned, 0, 0)

# status 2 (XC_NOT_CONVERGED) from a step means the step was completed but a
# Stokes solve stopped at its cap: raise with the step statistics
function check_step(status, st::StepStats)
    status == 2 && error("xcore_gb300: " * unsafe_string(ccall((:xc_last_error, LIB), Cstring, ())) *
                         " (unconverged solves: $(st.unconverged_solves))")
    check(status)
    return st
end

# one outer step of run! with `sweeps` Picard sweeps; returns the next dt
function step!(ctx::Context, step::Integer, dt, re, rs; sweeps = 3, solver::Symbol = :mixed, rtol = 1e-9)
    st = Ref(StepStats())
    status = ccall((:xc_step, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cdouble, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ref{SolverOpts}, Ref{StepStats}),
                   ctx.h, step, dt, sweeps, Matrix{Float64}(re), Matrix{Float64}(rs), step_solver_opts(solver, rtol), st)
    return check_step(status, st[]).dt_next
end

# one outer step of run! with the reference's Picard loop (src/run.jl:220-250) and
# its par.rtol, par.atol, par.maxit; returns (dt_next, sweeps)
function step_converge!(ctx::Context, step::Integer, dt, re, rs, par; solver::Symbol = :mixed, rtol = 1e-9)
    st = Ref(StepStats())
    status = ccall((:xc_step_converge, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Cdouble, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ref{SolverOpts},
                    Ref{StepStats}),
                   ctx.h, step, dt, par.rtol, par.atol, par.maxit, Matrix{Float64}(re), Matrix{Float64}(rs),
                   step_solver_opts(solver, rtol), st)
    s = check_step(status, st[])
    return (s.dt_next, Int(s.sweeps))
end

# ---- ensembles: independent contexts stepped together (xc_ensemble_*) ---------------
# every explicit stage of a Picard sweep one CUDA graph launch for all members,
# the Stokes solves on `threads` library threads (0: one per member); each
# member ends bit-identical to step! on it alone
mutable struct Ensemble
    h::Ptr{Cvoid}
    members::Vector{Context}
end

function Ensemble(members::Vector{Context}; threads::Integer = 0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    hs = Ptr{Cvoid}[m.h for m in members]
    check(ccall((:xc_ensemble_create, LIB), Cint, (Ptr{Ptr{Cvoid}}, Cint, Cint, Ref{Ptr{Cvoid}}),
                hs, length(hs), threads, h))
    e = Ensemble(h[], members)
    finalizer(x -> ccall((:xc_ensemble_destroy, LIB), Cint, (Ptr{Cvoid},), x.h), e)
    return e
end

# one time step of every member with `sweeps` Picard sweeps (steps[i], dts[i],
# draws re[i], rs[i]); returns the members' next dt
function step!(e::Ensemble, steps::AbstractVector{<:Integer}, dts::AbstractVector{<:Real}, re, rs;
               sweeps = 3, solver::Symbol = :mixed, rtol = 1e-9)
    n = length(e.members)
    st = Vector{StepStats}(undef, n)
    hre = [Matrix{Float64}(r) for r in re]
    hrs = [Matrix{Float64}(r) for r in rs]
    status = GC.@preserve hre hrs begin
        ccall((:xc_ensemble_step, LIB), Cint,
              (Ptr{Cvoid}, Ptr{Cint}, Ptr{Cdouble}, Cint, Ptr{Ptr{Cdouble}}, Ptr{Ptr{Cdouble}}, Ref{SolverOpts},
               Ptr{StepStats}),
              e.h, Cint.(steps), Cdouble.(dts), sweeps, [pointer(r) for r in hre], [pointer(r) for r in hrs],
              step_solver_opts(solver, rtol), st)
    end
    status == 2 && error("xcore_gb300: " * unsafe_string(ccall((:xc_last_error, LIB), Cstring, ())))
    check(status)
    return [s.dt_next for s in st]
end

# ---- call-site drop-in on CuArray-backed states -------------------------------------
# With CUDA.jl loaded and the reference's FluidState / PhaseState built on
# CuArrays (xcore_zeros with a CUDA backend, src/backend.jl:12-13), the methods
# below give run! (src/run.jl:204-275) the GPU path with its calls unchanged:
# each adds a method of the reference function for CuArray-backed states that
# binds the structs' arrays to a context field by field (xc_field_bind, zero
# copy; one context per PhaseState, cached) and calls the library.  The
# NoiseState stays on the host -- its MersenneTwister draws the white noise
# exactly as the reference does (noise.jl:154-157) -- while its time-evolving
# fields live in the context (download! / upload! move them for checkpoints).
using CUDA
using Random

const GPUFluid = xcore.FluidState{Float64,<:CuArray}
const GPUPhase = xcore.PhaseState{Float64,<:CuArray}
# Every positional argument below carries the reference's type at T = Float64:
# each method is then strictly more specific than the reference's own
# (a method that left grid, par, ... untyped would tie with it and make every
# call ambiguous).
const Grid64 = xcore.Grid{Float64}
const Par64 = xcore.Parameters{Float64}
const Scales64 = xcore.Scales{Float64}
const Noise64 = xcore.NoiseState{Float64}
const Res = xcore.StepResidual
const BOUND = IdDict{Any,Context}()
const BOUND_BC = IdDict{Any,NTuple{4,Int}}()   # (sds, top_cnv, bot_cnv, open_cnv) of each bound context
# the Stokes solver of the fluidmech! method below: the plain FP64 drop-in to
# relative residual 1e-10 (within 1e-8 of the reference's LU solution) by
# default; `XcoreGPU.CALLSITE_SOLVER[] = (:mixed, 1e-9)` selects the mixed
# FP32/FP64 solver (about 2.8x faster per step at 1024^2)
const CALLSITE_SOLVER = Ref{Tuple{Symbol,Float64}}((:fgmres64, 1e-10))

function bind!(ctx::Context, name::Symbol, a::CuArray)
    id = fieldid(name)
    id < 0 && return
    check(ccall((:xc_field_bind, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}), ctx.h, id,
                reinterpret(Ptr{Cvoid}, pointer(a))))
end

# the context whose fields are the arrays of (phase, fluid); created and bound
# on first use with the run's boundary keywords
function bound_context(phase::GPUPhase, fluid::GPUFluid, grid, par, scales; xBC = :periodic, zBC = :closed,
                       sds = -1, top_cnv = 1, bot_cnv = 1, open_cnv = false)
    get!(BOUND, phase) do
        BOUND_BC[phase] = (sds, top_cnv, bot_cnv, Int(open_cnv))
        ctx = Context(par, grid, scales; xBC, zBC, sds, top_cnv, bot_cnv, open_cnv)
        foreach_field((n, v) -> v isa CuArray && bind!(ctx, n, v), fluid, phase)
        ctx
    end
end
function bound_context(phase::GPUPhase)
    haskey(BOUND, phase) || error("XcoreGPU: no context bound to this PhaseState yet (call phsevo! or " *
                                  "fluidmech! with its grid, par and scales first)")
    return BOUND[phase]
end

function xcore.store_previous!(fluid::GPUFluid, phase::GPUPhase)
    ctx = bound_context(phase)
    store_previous!(ctx)
    # run! calls store_noise!(ns) right after (run.jl:206-207); the noise
    # history lives in the context, so it is stored here
    store_noise!(ctx)
end

xcore.snapshot!(res::Res, phase::GPUPhase, fluid::GPUFluid) = snapshot!(bound_context(phase))

function xcore.phsevo!(phase::GPUPhase, fluid::GPUFluid, grid::Grid64, par::Par64, scales::Scales64;
                       ADVN = par.ADVN, xBC = :periodic, zBC = :closed, a1, a2, a3, b1, b2, b3, dt, alpha = par.alpha)
    ctx = bound_context(phase, fluid, grid, par, scales; xBC, zBC)
    phsevo!(ctx; ADVN, a1, a2, a3, b1, b2, b3, dt, alpha)
end

function xcore.fluidmech!(fluid::GPUFluid, grid::Grid64, par::Par64; phase::GPUPhase, sds = -1, top_cnv = 1,
                          bot_cnv = 1, open_cnv = false, xBC = :periodic, zBC = :closed, dt = 1e32, a1 = 1.0,
                          a2 = 1.0, a3 = 0.0, b1 = 1.0, b2 = 0.0, b3 = 0.0)
    # run! calls phsevo! first in every sweep, which binds the context; the
    # Stokes boundary keywords are the context's (call bound_context with
    # them before run! when they are not the defaults)
    ctx = bound_context(phase)
    BOUND_BC[phase] == (sds, top_cnv, bot_cnv, Int(open_cnv)) ||
        error("XcoreGPU.fluidmech!: boundary keywords differ from the bound context's $(BOUND_BC[phase])")
    s = Ref{SolverStats}()
    check(ccall((:xc_fluidmech, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cdouble, Ref{SolverOpts}, Ref{SolverStats}),
                ctx.h, coefs(a1, a2, a3, b1, b2, b3), dt, step_solver_opts(CALLSITE_SOLVER[]...), s))
    return nothing
end

function xcore.noise!(ns::Noise64, phase::GPUPhase, grid::Grid64, par::Par64, scales::Scales64, dt::Real;
                      first_iter::Bool = true)
    ctx = bound_context(phase)
    if first_iter
        randn!(ns.rng, ns.re)
        randn!(ns.rng, ns.rs)
        noise!(ctx, dt; first_iter = true, re = ns.re, rs = ns.rs)
    else
        noise!(ctx, dt; first_iter = false)
    end
end

xcore.update_phase_velocities!(phase::GPUPhase, fluid::GPUFluid, ns::Noise64, grid::Grid64, par::Par64;
                               xBC = :periodic, zBC = :closed) =
    update_phase_velocities!(bound_context(phase))
xcore.update!(phase::GPUPhase, fluid::GPUFluid, grid::Grid64, par::Par64, scales::Scales64; xBC = :periodic,
              zBC = :closed) =
    update!(bound_context(phase))
function xcore.compute_resnorm(res::Res, phase::GPUPhase, fluid::GPUFluid, dt::Real)
    r = compute_resnorm(bound_context(phase), dt)
    # the reference's side effect on the StepResidual (src/diagnose.jl:67-69)
    if res.resnorm0 < r[1]
        res.resnorm0 = r[1] + 1e-32
    end
    return r
end
# record_history! (src/history.jl:101-222): the mass sums, boundary-flux
# integrals and the 58 field statistics come from the device
# (xc_conservation_sums, xc_history_stats, whose keys are the History field
# names); the rate shift, the BD2-integrated drift and the conservation
# errors are the reference's host arithmetic on them
function xcore.record_history!(hst::xcore.History{Float64}, time::Real, dt::Real, phase::GPUPhase,
                               fluid::GPUFluid, ns::Noise64, grid::Grid64, a1::Real = 1.0, a2::Real = 1.0,
                               a3::Real = 0.0, b1::Real = 1.0, b2::Real = 0.0, b3::Real = 0.0)
    ctx = bound_context(phase)
    hst.dsumBdtoo = hst.dsumBdto;  hst.dsumBdto = hst.dsumBdt
    hst.dsumMdtoo = hst.dsumMdto;  hst.dsumMdto = hst.dsumMdt
    hst.dsumXdtoo = hst.dsumXdto;  hst.dsumXdto = hst.dsumXdt
    push!(hst.time, Float64(time))
    push!(hst.dt, Float64(dt))
    sumB, sumM, sumX, sumGx, top_aX, bot_aX, top_aM, bot_aM, top_dX, bot_dX, top_dM, bot_dM = conservation_sums(ctx)
    push!(hst.sumB, sumB); push!(hst.sumM, sumM); push!(hst.sumX, sumX)
    hst.dsumBdt = (top_aX - bot_aX) + (top_aM - bot_aM) + (top_dX - bot_dX) + (top_dM - bot_dM)
    hst.dsumMdt = -sumGx + (top_aM - bot_aM) + (top_dM - bot_dM)
    hst.dsumXdt = +sumGx + (top_aX - bot_aX) + (top_dX - bot_dX)
    stp = length(hst.time)
    T = Float64
    drift(D, rate, rate_o, rate_oo) = stp >= 2 ?
        (T(a2) * D[stp - 1] + T(a3) * D[max(1, stp - 2)] + (T(b1) * rate + T(b2) * rate_o + T(b3) * rate_oo) * T(dt)) /
        T(a1) : zero(T)
    push!(hst.DB, drift(hst.DB, hst.dsumBdt, hst.dsumBdto, hst.dsumBdtoo))
    push!(hst.DM, drift(hst.DM, hst.dsumMdt, hst.dsumMdto, hst.dsumMdtoo))
    push!(hst.DX, drift(hst.DX, hst.dsumXdt, hst.dsumXdto, hst.dsumXdtoo))
    sumB0 = hst.sumB[1]
    push!(hst.EB, (sumB - hst.DB[stp] - sumB0) / sumB0)
    push!(hst.EM, (sumM - hst.DM[stp] - hst.sumM[1]) / sumB0)
    push!(hst.EX, (sumX - hst.DX[stp] - hst.sumX[1]) / sumB0)
    for (k, v) in history_stats(ctx)
        push!(getfield(hst, Symbol(k)), v)
    end
    return nothing
end

xcore.update_dt(phase::GPUPhase, fluid::GPUFluid, grid::Grid64, par::Par64, dt_prev::Real) =
    update_dt(bound_context(phase), dt_prev)

end # module
