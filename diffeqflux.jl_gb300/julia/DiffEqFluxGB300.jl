"""
    DiffEqFluxGB300

Julia host glue for libgbnde.so: routes `NeuralODE` (src/neural_de.jl:47-61),
`FFJORD` (src/ffjord.jl:138-178) and `multiple_shoot` (src/multiple_shooting.jl:36-94)
solves to the GB300 kernels through `ccall`, each with a
`ChainRulesCore.rrule` so that Zygote differentiates through the library's
adjoint (the role SciMLSensitivity's rrule on `solve` plays in the reference,
src/neural_de.jl:55-58, src/ffjord.jl:143).

Usage (drop-in for the reference's layer calls):

    using DiffEqFlux, DiffEqFluxGB300
    node = gb300(NeuralODE(Chain(Dense(64 => 256, tanh), Dense(256 => 256, tanh), Dense(256 => 64)),
                           (0f0, 1f0); saveat = range(0f0, 1f0, length = 20),
                           abstol = 1f-7, reltol = 1f-5), GB300Tsit5(:bf16))
    sol, st = node(u0, ps, st)          # sol::ODESolution, Array(sol) works
    gs = Zygote.gradient(p -> sum(abs2, Array(first(node(u0, p, st)))), ps)

    cnf = gb300(FFJORD(Chain(Dense(2 => 32, tanh), Dense(32 => 2)), (0f0, 1f0), (2,)), GB300Tsit5(:fp32))
    (logpx, _, _), _ = cnf(x, ps_cnf, st_cnf)

    loss, preds = multiple_shoot(p, ode_data, tsteps, model, gb300_mse, GB300Tsit5(:fp32), group_size;
                                 continuity_term = 100)

Only Chain([WrappedFunction(x -> x.^3),] Dense...) models with tanh /
softplus / identity activations are accepted; anything else throws (there is
no CPU fallback). Parameters are passed as the flat ComponentArray vector.
"""
module DiffEqFluxGB300

using ChainRulesCore, ComponentArrays, DiffEqFlux, Lux, SciMLBase, SciMLSensitivity
using Distributions: logpdf

export GB300Tsit5, gb300, gb300_train_step!, gb300_autotune!, gb300_mse, gb300_sse

const libgbnde = joinpath(@__DIR__, "..", "gbnde", "libgbnde.so")

# ---- C ABI mirrors (include/gbnde.h) -------------------------------------------------
const MAX_LAYERS = 8

struct MlpDesc
    nlayers::Cint
    dims::NTuple{MAX_LAYERS + 1, Cint}
    act::NTuple{MAX_LAYERS, Cint}
    cube_input::Cint
    time_input::Cint
end

struct SolveDesc
    t0::Cdouble
    t1::Cdouble
    abstol::Cdouble
    reltol::Cdouble
    dt0::Cdouble
    dtmin::Cdouble
    maxiters::Clonglong
    saveat::Ptr{Cdouble}
    nsave::Cint
    sensealg::Cint
    flags::Cint
end

struct Segment
    t0::Cdouble
    t1::Cdouble
    save_off::Cint
    nsave::Cint
end

mutable struct Stats
    nf::Clonglong
    naccept::Clonglong
    nreject::Clonglong
    nf_recompute::Clonglong
    nf_adj::Clonglong
    naccept_adj::Clonglong
    nreject_adj::Clonglong
    retcode::Cint
    retcode_adj::Cint
    t_final::Cdouble
    nf_adj_vjp::Clonglong
    fwd_path::Cint
    adj_path::Cint
    Stats() = new(0, 0, 0, 0, 0, 0, 0, 0, 0, 0.0, 0, 0, 0)
end

const RETCODES = (SciMLBase.ReturnCode.Success, SciMLBase.ReturnCode.MaxIters,
                  SciMLBase.ReturnCode.DtLessThanMin, SciMLBase.ReturnCode.Unstable,
                  SciMLBase.ReturnCode.Failure)

check(rc) = rc == 0 || error("gbnde error $rc: " *
                             unsafe_string(ccall((:gbnde_last_error, libgbnde), Cstring, ())))

# ---- algorithm marker -------------------------------------------------------------------
"""`GB300Tsit5(precision = :bf16)` -- Tsit5 on the GB300 kernels (:bf16 or :fp32)."""
struct GB300Tsit5 <: SciMLBase.AbstractODEAlgorithm
    precision::Symbol
end
GB300Tsit5() = GB300Tsit5(:bf16)

_act(f) = f === identity ? 0 : f === tanh || f === Lux.tanh_fast ? 1 :
          f === Lux.softplus ? 2 : error("unsupported activation $f")

function mlp_desc(model::Chain; time_input = false)
    layers = collect(values(model.layers))
    cube = layers[1] isa WrappedFunction
    dense = filter(l -> l isa Dense, layers)
    dims = Cint[dense[1].in_dims; [d.out_dims for d in dense]...]
    acts = Cint[_act(d.activation) for d in dense]
    pad(v, n) = ntuple(i -> i <= length(v) ? v[i] : Cint(0), n)
    MlpDesc(length(dense), pad(dims, MAX_LAYERS + 1), pad(acts, MAX_LAYERS), cube, time_input)
end

# One library context per (model, precision); finalised with the Julia object.
# `gen` counts the solves run on it: the library's backward differentiates the
# context's LAST solve, so a pullback whose solve is no longer the last one
# solves it again first (a layer called twice before the gradient is taken).
mutable struct Ctx
    h::Ptr{Cvoid}
    nparams::Int
    gen::Int
    stats::Stats
end
function Ctx(model::Chain, precision::Symbol; time_input = false)
    d = Ref(mlp_desc(model; time_input))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gbnde_create, libgbnde), Cint, (Ptr{Ptr{Cvoid}}, Ref{MlpDesc}, Cint, Cint),
                h, d, precision === :bf16 ? 1 : 0, 0))
    c = Ctx(h[], Int(ccall((:gbnde_nparams, libgbnde), Csize_t, (Ptr{Cvoid},), h[])), 0, Stats())
    finalizer(x -> ccall((:gbnde_destroy, libgbnde), Cvoid, (Ptr{Cvoid},), x.h), c)
    c
end

const CTXS = IdDict{Any, Ctx}()
ctx_for(model, prec; time_input = false) =
    get!(() -> Ctx(model, prec; time_input), CTXS, (model, prec, time_input))

set_params!(ctx::Ctx, p) = check(ccall((:gbnde_set_params, libgbnde), Cint, (Ptr{Cvoid}, Ptr{Float32}, Csize_t),
                                       ctx.h, p, length(p)))

sensecode(s) = s isa BacksolveAdjoint ? 1 : s isa InterpolatingAdjoint ? 0 :
               (s isa QuadratureAdjoint || s isa GaussAdjoint) ? 2 :
               error("GB300 supports InterpolatingAdjoint, BacksolveAdjoint, QuadratureAdjoint and GaussAdjoint")

# ---- the differentiable NeuralODE solve -------------------------------------------------
"""
    gb300_solve(u0, p, ctx, tspan, saveat, abstol, reltol, sensealg, flags) -> Array (S, B, nsave)

The saved states of `solve(ODEProblem{false}(dudt, u0, tspan, p), Tsit5(); saveat,
abstol, reltol)` (src/neural_de.jl:52-58) on the GB300 kernels. `flags =
GBNDE_FLAG_FP32_TIME` keeps t and dt in Float32 (the FP32 form with a Float32
tspan). The solve's counters and retcode are left in `ctx.stats`.
"""
const GBNDE_FLAG_FP32_TIME = Cint(1)
function gb300_solve(u0::AbstractMatrix{Float32}, p::AbstractVector{Float32}, ctx::Ctx, tspan,
                     saveat::Vector{Float64}, abstol, reltol, sensealg, flags = Cint(0))
    S, B = size(u0)
    set_params!(ctx, p)
    out = Array{Float32}(undef, S, B, length(saveat))
    st = Stats()
    GC.@preserve saveat begin
        d = Ref(SolveDesc(tspan[1], tspan[2], abstol, reltol, 0, 0, 100000, pointer(saveat),
                          length(saveat), sensecode(sensealg), flags))
        check(ccall((:gbnde_forward, libgbnde), Cint,
                    (Ptr{Cvoid}, Ref{SolveDesc}, Cint, Cint, Ptr{Float32}, Ptr{Float32}, Ref{Stats}),
                    ctx.h, d, S, B, Matrix{Float32}(u0), out, st))
    end
    ctx.gen += 1
    ctx.stats = st
    out
end

# Cotangent of the saved states, whatever shape Zygote hands back: an array
# (from Array(sol) or a 3-d slice), a tangent of the ODESolution or of its
# `u` field (one entry per save, each S x B or S), or zero.
function _saveat_cotangent(Δ, S, B, ns)
    Δ = unthunk(Δ)
    out = zeros(Float32, S, B, ns)
    Δ isa AbstractZero && return out
    if Δ isa AbstractArray && eltype(Δ) <: Number
        out .= reshape(Float32.(Δ), S, B, ns)
        return out
    end
    u = Δ isa AbstractVector ? Δ : unthunk(hasproperty(Δ, :u) ? getproperty(Δ, :u) : Δ)
    u isa AbstractZero && return out
    for (i, ui) in enumerate(u)
        ui = unthunk(ui)
        ui isa AbstractZero && continue
        out[:, :, i] .= reshape(Float32.(ui), S, B)
    end
    out
end

function ChainRulesCore.rrule(::typeof(gb300_solve), u0, p, ctx, tspan, saveat, abstol, reltol,
                              sensealg, flags = Cint(0))
    out = gb300_solve(u0, p, ctx, tspan, saveat, abstol, reltol, sensealg, flags)
    gen = ctx.gen
    retcode = ctx.stats.retcode
    function gb300_solve_pullback(Δ)
        retcode == 0 || error("cannot differentiate a failed GB300 solve (retcode $retcode)")
        S, B = size(u0)
        # another solve ran on the context since: solve this one again
        # (deterministic, so the checkpoints are the ones `out` came from)
        ctx.gen == gen || gb300_solve(u0, p, ctx, tspan, saveat, abstol, reltol, sensealg, flags)
        du0 = Matrix{Float32}(undef, S, B)
        dp = Vector{Float32}(undef, length(p))
        bst = Stats()
        check(ccall((:gbnde_backward, libgbnde), Cint,
                    (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Ref{Stats}),
                    ctx.h, _saveat_cotangent(Δ, S, B, length(saveat)), du0, dp, bst))
        (NoTangent(), du0, dp, NoTangent(), NoTangent(), NoTangent(), NoTangent(), NoTangent(),
         NoTangent(), NoTangent())
    end
    out, gb300_solve_pullback
end

# The ODESolution the reference returns (`Array(sol)`, `sol.u`, `sol.t`,
# `sol.retcode`, src/neural_de.jl:55-60), built from the saved states; its
# rrule unwraps an ODESolution-shaped tangent back to the S x B x nsave array.
function _build_sol(prob, alg, saveat, out, vec_input::Bool, retcode)
    us = [vec_input ? out[:, 1, i] : out[:, :, i] for i in axes(out, 3)]
    SciMLBase.build_solution(prob, alg, saveat, us; retcode)
end
function ChainRulesCore.rrule(::typeof(_build_sol), prob, alg, saveat, out, vec_input, retcode)
    sol = _build_sol(prob, alg, saveat, out, vec_input, retcode)
    S, B, ns = size(out)
    _build_sol_pullback(Δ) = (NoTangent(), NoTangent(), NoTangent(), NoTangent(),
                              _saveat_cotangent(Δ, S, B, ns), NoTangent(), NoTangent())
    sol, _build_sol_pullback
end

# ---- NeuralODE on the GB300 path (src/neural_de.jl:47-61) --------------------------------
# Accepted steps (t_n, h_n) of the context's last forward solve.
function forward_steps(ctx::Ctx)
    n = ccall((:gbnde_forward_steps, libgbnde), Clonglong, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Clonglong),
              ctx.h, C_NULL, C_NULL, 0)
    t = zeros(Cdouble, n)
    h = zeros(Cdouble, n)
    ccall((:gbnde_forward_steps, libgbnde), Clonglong, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Clonglong),
          ctx.h, t, h, n)
    t, h
end

function (n::NeuralODE)(x, p, st, alg::GB300Tsit5)
    kw = Dict(n.kwargs)
    ctx = ctx_for(n.model, alg.precision)
    sense = get(kw, :sensealg, InterpolatingAdjoint(; autojacvec = ZygoteVJP()))
    u0 = x isa AbstractVector ? reshape(x, :, 1) : x
    # a Float32 tspan keeps t and dt in Float32, as the reference's integrator does
    flags = (eltype(n.tspan) === Float32 && alg.precision === :fp32) ? GBNDE_FLAG_FP32_TIME : Cint(0)
    abstol, reltol = get(kw, :abstol, 1e-6), get(kw, :reltol, 1e-3)
    everystep = get(kw, :save_everystep, !haskey(kw, :saveat))
    saveat = if everystep
        # every accepted step: the save points never change the step sizes
        # (only the end of the span clips a step), so a first solve gives the
        # steps and the solve saving at their ends takes the same steps
        ChainRulesCore.@ignore_derivatives begin
            gb300_solve(Float32.(u0), Float32.(collect(p)), ctx, Float64.(n.tspan), Float64[n.tspan[2]],
                        abstol, reltol, sense, flags)
            ts, _ = forward_steps(ctx)
            ends = length(ts) > 0 ? [ts[2:end]; Float64(n.tspan[2])] : [Float64(n.tspan[2])]
            get(kw, :save_start, true) ? [Float64(n.tspan[1]); ends] : ends
        end
    else
        Float64.(collect(get(kw, :saveat, [n.tspan[2]])))
    end
    out = gb300_solve(Float32.(u0), Float32.(collect(p)), ctx, Float64.(n.tspan), saveat, abstol, reltol, sense,
                      flags)
    retcode = ChainRulesCore.@ignore_derivatives RETCODES[ctx.stats.retcode + 1]
    prob = ChainRulesCore.@ignore_derivatives ODEProblem{false}((u, p, t) -> u, x, n.tspan, p)
    _build_sol(prob, alg, saveat, out, x isa AbstractVector, retcode), st
end

# ---- FFJORD on the GB300 path (src/ffjord.jl:138-178) ------------------------------------
"""
    gb300_ffjord(x, p, ctx, tspan, abstol, reltol, noise) -> (logpx (1 x B), z(t1) (d x B))

`__forward_ffjord` with the standard-normal base on the kernels: the augmented
system [z; delta_logp] solved from (x, 0) over tspan, end state only. `noise`:
d x B Hutchinson directions fixed for the solve, or `nothing` for the exact
trace (monte_carlo = false).
"""
function gb300_ffjord(x::AbstractMatrix{Float32}, p::AbstractVector{Float32}, ctx::Ctx, tspan, abstol, reltol,
                      noise)
    d, B = size(x)
    set_params!(ctx, p)
    logpx = Vector{Float32}(undef, B)
    zT = Matrix{Float32}(undef, d, B)
    st = Stats()
    sv = Float64[tspan[2]]
    GC.@preserve sv noise begin
        sd = Ref(SolveDesc(tspan[1], tspan[2], abstol, reltol, 0, 0, 100000, pointer(sv), 1, 0, 0))
        nz = noise === nothing ? Ptr{Float32}(C_NULL) : pointer(noise)
        check(ccall((:gbnde_ffjord_forward, libgbnde), Cint,
                    (Ptr{Cvoid}, Ref{SolveDesc}, Cint, Cint, Ptr{Float32}, Ptr{Float32}, Ptr{Float32},
                     Ptr{Float32}, Ref{Stats}),
                    ctx.h, sd, d, B, Matrix{Float32}(x), nz, logpx, zT, st))
    end
    ctx.gen += 1
    ctx.stats = st
    reshape(logpx, 1, B), zT
end

function ChainRulesCore.rrule(::typeof(gb300_ffjord), x, p, ctx, tspan, abstol, reltol, noise)
    logpx, zT = gb300_ffjord(x, p, ctx, tspan, abstol, reltol, noise)
    gen = ctx.gen
    function gb300_ffjord_pullback(Δ)
        d, B = size(x)
        Δl, Δz = unthunk(Δ[1]), unthunk(Δ[2])
        gl = Δl isa AbstractZero ? zeros(Float32, B) : vec(Float32.(Δl))
        gz = Δz isa AbstractZero ? nothing : Matrix{Float32}(Δz)
        ctx.gen == gen || gb300_ffjord(x, p, ctx, tspan, abstol, reltol, noise)
        dx = Matrix{Float32}(undef, d, B)
        dp = Vector{Float32}(undef, length(p))
        bst = Stats()
        GC.@preserve gz begin
            check(ccall((:gbnde_ffjord_backward, libgbnde), Cint,
                        (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Ref{Stats}),
                        ctx.h, gl, gz === nothing ? Ptr{Float32}(C_NULL) : pointer(gz), dx, dp, bst))
        end
        (NoTangent(), dx, dp, NoTangent(), NoTangent(), NoTangent(), NoTangent(), NoTangent())
    end
    (logpx, zT), gb300_ffjord_pullback
end

"""
    gb300_ffjord_reg(x, p, ctx, tspan, abstol, reltol, noise, exact)
        -> (logpx (1 x B), z(t1) (d x B), λ₁ (1 x B), λ₂ (1 x B))

`regularize = true` (src/ffjord.jl:131-135): two more rows integrate |f|^2 and
|eᵀJ| from 0; λ₁ and λ₂ are their values at t1. `noise` (d x B) is the e of
|eᵀJ| and, unless `exact`, the Hutchinson direction.
"""
function gb300_ffjord_reg(x::AbstractMatrix{Float32}, p::AbstractVector{Float32}, ctx::Ctx, tspan, abstol,
                          reltol, noise::AbstractMatrix{Float32}, exact::Bool)
    d, B = size(x)
    set_params!(ctx, p)
    logpx = Vector{Float32}(undef, B)
    zT = Matrix{Float32}(undef, d, B)
    rf = Vector{Float32}(undef, B)
    rj = Vector{Float32}(undef, B)
    st = Stats()
    sv = Float64[tspan[2]]
    GC.@preserve sv noise begin
        sd = Ref(SolveDesc(tspan[1], tspan[2], abstol, reltol, 0, 0, 100000, pointer(sv), 1, 0, 0))
        check(ccall((:gbnde_ffjord_forward_reg, libgbnde), Cint,
                    (Ptr{Cvoid}, Ref{SolveDesc}, Cint, Cint, Ptr{Float32}, Ptr{Float32}, Cint, Ptr{Float32},
                     Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Ref{Stats}),
                    ctx.h, sd, d, B, Matrix{Float32}(x), pointer(noise), Cint(exact), logpx, zT, rf, rj, st))
    end
    ctx.gen += 1
    ctx.stats = st
    reshape(logpx, 1, B), zT, reshape(rf, 1, B), reshape(rj, 1, B)
end

function ChainRulesCore.rrule(::typeof(gb300_ffjord_reg), x, p, ctx, tspan, abstol, reltol, noise, exact)
    out = gb300_ffjord_reg(x, p, ctx, tspan, abstol, reltol, noise, exact)
    gen = ctx.gen
    function gb300_ffjord_reg_pullback(Δ)
        d, B = size(x)
        Δl, Δz, Δf, Δj = unthunk(Δ[1]), unthunk(Δ[2]), unthunk(Δ[3]), unthunk(Δ[4])
        gl = Δl isa AbstractZero ? zeros(Float32, B) : vec(Float32.(Δl))
        gz = Δz isa AbstractZero ? nothing : Matrix{Float32}(Δz)
        gf = Δf isa AbstractZero ? nothing : vec(Float32.(Δf))
        gj = Δj isa AbstractZero ? nothing : vec(Float32.(Δj))
        ctx.gen == gen || gb300_ffjord_reg(x, p, ctx, tspan, abstol, reltol, noise, exact)
        dx = Matrix{Float32}(undef, d, B)
        dp = Vector{Float32}(undef, length(p))
        bst = Stats()
        ptr(a) = a === nothing ? Ptr{Float32}(C_NULL) : pointer(a)
        GC.@preserve gz gf gj begin
            check(ccall((:gbnde_ffjord_backward_reg, libgbnde), Cint,
                        (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32},
                         Ptr{Float32}, Ref{Stats}),
                        ctx.h, gl, ptr(gz), ptr(gf), ptr(gj), dx, dp, bst))
        end
        (NoTangent(), dx, dp, NoTangent(), NoTangent(), NoTangent(), NoTangent(), NoTangent(), NoTangent())
    end
    out, gb300_ffjord_reg_pullback
end

function _ffjord_forward(n::FFJORD, x::AbstractMatrix, ps, st, alg::GB300Tsit5)
    (; regularize, monte_carlo) = st
    regularize && return _ffjord_forward_reg(n, x, ps, st, alg)
    d, B = size(x)
    ctx = ctx_for(n.model, alg.precision)
    kw = Dict(n.kwargs)
    # Hutchinson directions: Gaussian as the reference draws them
    # (src/ffjord.jl:92), but one draw per sample for the whole solve
    noise = monte_carlo ? ChainRulesCore.@ignore_derivatives(randn(Float32, d, B)) : nothing
    logpx_std, zT = gb300_ffjord(Float32.(x), Float32.(collect(ps)), ctx, Float64.(n.tspan),
                                 get(kw, :abstol, 1e-6), get(kw, :reltol, 1e-3), noise)
    T = Float32
    logpz_std = -sum(abs2, zT; dims = 1) / T(2) .- T(d / 2 * log(2π))
    delta_logp = logpz_std .- logpx_std
    logpx = n.basedist === nothing ? logpx_std : reshape(logpdf(n.basedist, zT), 1, B) .- delta_logp
    (logpx, delta_logp, delta_logp), st
end

# regularize = true: (logpx, λ₁, λ₂) with λ₁, λ₂ the two regulariser rows at t1.
# (The reference selects λ₁ and λ₂ along the batch dimension of the end state,
# src/ffjord.jl:164-166, i.e. batch columns; its tests read only logpx.)
function _ffjord_forward_reg(n::FFJORD, x::AbstractMatrix, ps, st, alg::GB300Tsit5)
    d, B = size(x)
    ctx = ctx_for(n.model, alg.precision)
    kw = Dict(n.kwargs)
    noise = ChainRulesCore.@ignore_derivatives(randn(Float32, d, B))
    logpx_std, zT, λ₁, λ₂ = gb300_ffjord_reg(Float32.(x), Float32.(collect(ps)), ctx, Float64.(n.tspan),
                                             get(kw, :abstol, 1e-6), get(kw, :reltol, 1e-3), noise,
                                             !st.monte_carlo)
    T = Float32
    logpz_std = -sum(abs2, zT; dims = 1) / T(2) .- T(d / 2 * log(2π))
    delta_logp = logpz_std .- logpx_std
    logpx = n.basedist === nothing ? logpx_std : reshape(logpdf(n.basedist, zT), 1, B) .- delta_logp
    (logpx, λ₁, λ₂), st
end

# ---- multiple shooting on the GB300 path (src/multiple_shooting.jl:36-94) ---------------
"""`gb300_mse(u, û)` / `gb300_sse(u, û)`: mean / sum of squares. Passed as the
`loss_function` of `multiple_shoot` together with the default continuity loss,
they put the whole loss in one device kernel (gbnde_multishoot_loss)."""
gb300_mse(u, uh) = sum(abs2, u .- uh) / length(u)
gb300_sse(u, uh) = sum(abs2, u .- uh)

# Segment table of multiple_shoot's groups (group_ranges, src/multiple_shooting.jl:231-239).
function _ms_layout(ode_data::AbstractMatrix, tsteps, group_size)
    ranges = DiffEqFlux.group_ranges(size(ode_data, 2), group_size)
    segs = Segment[]
    saveat = Float64[]
    for rg in ranges
        push!(segs, Segment(tsteps[first(rg)], tsteps[last(rg)], length(saveat), length(rg)))
        append!(saveat, Float64.(tsteps[rg]))
    end
    nxt = Cint[i < length(ranges) ? i : -1 for i in 1:length(ranges)]   # 0-based successor
    u0s = Matrix{Float32}(ode_data[:, first.(ranges)])
    data = Matrix{Float32}(reduce(hcat, [ode_data[:, rg] for rg in ranges]))
    ranges, segs, saveat, nxt, u0s, data
end

function _ms_forward(ctx::Ctx, p, segs, saveat, u0s, abstol, reltol, maxiters)
    S, nseg = size(u0s)
    set_params!(ctx, Float32.(collect(p)))
    usave = Matrix{Float32}(undef, S, length(saveat))
    ret = zeros(Cint, nseg)
    st = Stats()
    check(ccall((:gbnde_multishoot_forward, libgbnde), Cint,
                (Ptr{Cvoid}, Cint, Cint, Ptr{Segment}, Ptr{Cdouble}, Cint, Ptr{Float32}, Cdouble, Cdouble,
                 Clonglong, Ptr{Float32}, Ptr{Cint}, Ref{Stats}),
                ctx.h, S, nseg, segs, saveat, length(saveat), u0s, abstol, reltol, maxiters, usave, ret, st))
    ctx.gen += 1
    ctx.stats = st
    usave, ret
end

function _ms_grad(ctx::Ctx, dL_dusave, nparams, nseg, S)
    dp = Vector{Float32}(undef, nparams)
    bst = Stats()
    check(ccall((:gbnde_multishoot_backward, libgbnde), Cint,
                (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Ref{Stats}),
                ctx.h, dL_dusave === nothing ? Ptr{Float32}(C_NULL) : dL_dusave, Ptr{Float32}(C_NULL), dp, bst))
    dp
end

# all groups' predictions (S x nsave_total, packed like the saves): the
# general route, where Zygote differentiates the user's loss in Julia
function gb300_ms_predict(p, ctx, segs, saveat, u0s, abstol, reltol, maxiters)
    _ms_forward(ctx, p, segs, saveat, u0s, abstol, reltol, maxiters)
end
function ChainRulesCore.rrule(::typeof(gb300_ms_predict), p, ctx, segs, saveat, u0s, abstol, reltol, maxiters)
    usave, ret = _ms_forward(ctx, p, segs, saveat, u0s, abstol, reltol, maxiters)
    gen = ctx.gen
    function gb300_ms_predict_pullback(Δ)
        Δu = unthunk(Δ[1])
        Δu isa AbstractZero && return (NoTangent(), ZeroTangent(), ntuple(_ -> NoTangent(), 7)...)
        all(==(0), ret) || error("cannot differentiate multiple shooting with a failed group")
        ctx.gen == gen || _ms_forward(ctx, p, segs, saveat, u0s, abstol, reltol, maxiters)
        dp = _ms_grad(ctx, Matrix{Float32}(Δu), length(p), length(segs), size(u0s, 1))
        (NoTangent(), dp, ntuple(_ -> NoTangent(), 7)...)
    end
    (usave, ret), gb300_ms_predict_pullback
end

# the fused route: loss and continuity terms in one kernel, the adjoint from
# the cotangent it leaves on the device
function gb300_ms_fused_loss(p, ctx, segs, saveat, u0s, data, nxt, kind, cont, abstol, reltol, maxiters)
    usave, ret = _ms_forward(ctx, p, segs, saveat, u0s, abstol, reltol, maxiters)
    all(==(0), ret) || return Inf, usave, ret
    l = Ref{Cdouble}(0)
    check(ccall((:gbnde_multishoot_loss, libgbnde), Cint,
                (Ptr{Cvoid}, Ptr{Float32}, Ptr{Cint}, Cint, Cdouble, Ref{Cdouble}),
                ctx.h, data, nxt, kind, cont, l))
    l[], usave, ret
end
function ChainRulesCore.rrule(::typeof(gb300_ms_fused_loss), p, ctx, segs, saveat, u0s, data, nxt, kind, cont,
                              abstol, reltol, maxiters)
    out = gb300_ms_fused_loss(p, ctx, segs, saveat, u0s, data, nxt, kind, cont, abstol, reltol, maxiters)
    gen = ctx.gen
    function gb300_ms_fused_pullback(Δ)
        Δl = unthunk(Δ[1])
        Δl isa AbstractZero && return (NoTangent(), ZeroTangent(), ntuple(_ -> NoTangent(), 11)...)
        isfinite(out[1]) || error("cannot differentiate multiple shooting with a failed group")
        ctx.gen == gen || gb300_ms_fused_loss(p, ctx, segs, saveat, u0s, data, nxt, kind, cont, abstol, reltol,
                                              maxiters)
        dp = _ms_grad(ctx, nothing, length(p), length(segs), size(u0s, 1))
        (NoTangent(), Float32(Δl) .* dp, ntuple(_ -> NoTangent(), 11)...)
    end
    out, gb300_ms_fused_pullback
end

"""
    multiple_shoot(p, ode_data, tsteps, model::Lux.Chain, loss_function, [continuity_loss],
                   GB300Tsit5(...), group_size; continuity_term = 100, abstol, reltol, maxiters)
        -> (loss, group_predictions)

The reference's `multiple_shoot` (src/multiple_shooting.jl:36-94) with the
GB300 solver: every group solved from its first data point with its own
adaptive controller, all groups in one kernel launch; Inf loss when a group
fails (:66-67). `model` stands in for the reference's `prob` (the right-hand
side must be a supported Lux Chain). `loss_function = gb300_mse / gb300_sse`
with the default continuity loss runs the loss on the device; any other loss
function is differentiated by Zygote in Julia over the predictions.
"""
function DiffEqFlux.multiple_shoot(p, ode_data::AbstractMatrix, tsteps, model::Lux.Chain, loss_function::F,
                                   continuity_loss::C, solver::GB300Tsit5, group_size::Integer;
                                   continuity_term::Real = 100, abstol = 1e-6, reltol = 1e-3,
                                   maxiters = 100000) where {F, C}
    datasize = size(ode_data, 2)
    (group_size < 2 || group_size > datasize) &&
        throw(DomainError(group_size, "group_size can't be < 2 or > number of data points"))
    ctx = ctx_for(model, solver.precision)
    ranges, segs, saveat, nxt, u0s, data = ChainRulesCore.@ignore_derivatives _ms_layout(ode_data, tsteps, group_size)
    slices(usave) = [usave[:, (segs[i].save_off + 1):(segs[i].save_off + segs[i].nsave)] for i in eachindex(segs)]
    kind = loss_function === gb300_mse ? Cint(1) : loss_function === gb300_sse ? Cint(0) : Cint(-1)
    if kind >= 0 && continuity_loss === DiffEqFlux._default_continuity_loss
        l, usave, ret = gb300_ms_fused_loss(p, ctx, segs, saveat, u0s, data, nxt, kind, Float64(continuity_term),
                                            abstol, reltol, maxiters)
        return l, ChainRulesCore.@ignore_derivatives(slices(usave))
    end
    usave, ret = gb300_ms_predict(p, ctx, segs, saveat, u0s, abstol, reltol, maxiters)
    preds = slices(usave)
    all(==(0), ret) || return Inf, preds
    loss = 0
    for (i, rg) in enumerate(ranges)
        u = ode_data[:, rg]
        loss += loss_function(u, preds[i])
        if i > 1
            loss += continuity_term * continuity_loss(preds[i - 1][:, end], u[:, 1])
        end
    end
    loss, preds
end

function DiffEqFlux.multiple_shoot(p, ode_data::AbstractMatrix, tsteps, model::Lux.Chain, loss_function::F,
                                   solver::GB300Tsit5, group_size::Integer; kwargs...) where {F}
    DiffEqFlux.multiple_shoot(p, ode_data, tsteps, model, loss_function, DiffEqFlux._default_continuity_loss,
                              solver, group_size; kwargs...)
end

# ---- one Adam training iteration on the device (gbnde_train_step) ------------------------
struct AdamDesc
    lr::Cdouble
    beta1::Cdouble
    beta2::Cdouble
    eps::Cdouble
end

"""
    gb300_train_step!(ctx, tspan, saveat, abstol, reltol, u0, target, p, m, v, step;
                      lr = 1e-3, beta1 = 0.9, beta2 = 0.999, eps = 1e-8, loss = :mse) -> (loss, stats)

One iteration of `Optimization.solve(optprob, OptimizationOptimisers.Adam(lr))`
(docs/src/examples/neural_ode.md:66-70) for a NeuralODE with an MSE/SSE loss at
the save points, entirely on the GPU: `u0`, `target`, `p`, `m`, `v` are
`CuArray{Float32}` (CUDA.jl), `p`, `m`, `v` updated in place.
"""
function gb300_train_step!(ctx::Ctx, tspan, saveat::Vector{Float64}, abstol, reltol, u0, target, p, m, v,
                           step::Integer; lr = 1e-3, beta1 = 0.9, beta2 = 0.999, eps = 1e-8, loss = :mse,
                           graph = false)
    S, B = size(u0)
    opt = Ref(AdamDesc(lr, beta1, beta2, eps))
    l = Ref{Cdouble}(0)
    st = Stats()
    g = Ref{Cint}(0)
    GC.@preserve saveat begin
        d = Ref(SolveDesc(tspan[1], tspan[2], abstol, reltol, 0, 0, 100000, pointer(saveat),
                          length(saveat), 0, 0))
        if graph  # replayed as one CUDA graph from the second call on
            check(ccall((:gbnde_graph_train_step, libgbnde), Cint,
                        (Ptr{Cvoid}, Ref{SolveDesc}, Cint, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ref{AdamDesc},
                         Clonglong, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{Cdouble}, Ref{Stats}, Ref{Cint}),
                        ctx.h, d, S, B, pointer(u0), pointer(target), loss === :mse ? 1 : 0, opt, step,
                        pointer(p), pointer(m), pointer(v), l, st, g))
        else
            check(ccall((:gbnde_train_step, libgbnde), Cint,
                        (Ptr{Cvoid}, Ref{SolveDesc}, Cint, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ref{AdamDesc},
                         Clonglong, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{Cdouble}, Ref{Stats}),
                        ctx.h, d, S, B, pointer(u0), pointer(target), loss === :mse ? 1 : 0, opt, step,
                        pointer(p), pointer(m), pointer(v), l, st))
        end
    end
    l[], st
end

"""
    gb300_autotune!(ctx, tspan, saveat, abstol, reltol, u0) -> (forward_rows, adjoint_rows)

Times the FP32 kernels at each rows-per-tile choice on `u0`'s shape
(`CuArray{Float32}`, S x B) and keeps the fastest in `ctx` for later solves.
"""
function gb300_autotune!(ctx::Ctx, tspan, saveat::Vector{Float64}, abstol, reltol, u0)
    S, B = size(u0)
    tiles = zeros(Cint, 2)
    GC.@preserve saveat begin
        d = Ref(SolveDesc(tspan[1], tspan[2], abstol, reltol, 0, 0, 100000, pointer(saveat),
                          length(saveat), 0, 0))
        check(ccall((:gbnde_autotune, libgbnde), Cint,
                    (Ptr{Cvoid}, Ref{SolveDesc}, Cint, Cint, Ptr{Cvoid}, Ptr{Cint}),
                    ctx.h, d, S, B, pointer(u0), tiles))
    end
    Int(tiles[1]), Int(tiles[2])
end

# A layer routed to the GB300 kernels keeps the reference's `(layer)(x, p, st)`
# call: `gb300(NeuralODE(...))` wraps it without touching DiffEqFlux's methods.
struct GB300Layer{L}
    layer::L
    alg::GB300Tsit5
end
gb300(layer, alg::GB300Tsit5 = GB300Tsit5()) = GB300Layer(layer, alg)
(g::GB300Layer{<:NeuralODE})(x, p, st) = g.layer(x, p, st, g.alg)
(g::GB300Layer{<:FFJORD})(x, ps, st) = _ffjord_forward(g.layer, x, ps, st, g.alg)

end # module
