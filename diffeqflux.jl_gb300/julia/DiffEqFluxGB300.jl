"""
    DiffEqFluxGB300

Julia host glue for libgbnde.so: routes `NeuralODE`, `FFJORD` and
`multiple_shoot` solves to the GB300 kernels through `ccall`, with a
`ChainRulesCore.rrule` so that Zygote differentiates through the library's
adjoint (the role SciMLSensitivity's rrule on `solve` plays in the reference,
src/neural_de.jl:55-58).

Usage (drop-in for the reference's layer calls):

    using DiffEqFlux, DiffEqFluxGB300
    node = gb300(NeuralODE(Chain(Dense(64 => 256, tanh), Dense(256 => 256, tanh), Dense(256 => 64)),
                           (0f0, 1f0); saveat = range(0f0, 1f0, length = 20),
                           abstol = 1f-7, reltol = 1f-5), GB300Tsit5(:bf16))
    sol, st = node(u0, ps, st)          # sol::ODESolution, Array(sol) works
    gs = Zygote.gradient(p -> sum(abs2, Array(first(node(u0, p, st)))), ps)

Only Chain([WrappedFunction(x -> x.^3),] Dense...) models with tanh /
softplus / identity activations are accepted; anything else throws (there is
no CPU fallback). Parameters are passed as the flat ComponentArray vector.
"""
module DiffEqFluxGB300

using ChainRulesCore, ComponentArrays, DiffEqFlux, Lux, SciMLBase, SciMLSensitivity

export GB300Tsit5, gb300, gb300_train_step!, gb300_autotune!

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
mutable struct Ctx
    h::Ptr{Cvoid}
    nparams::Int
end
function Ctx(model::Chain, precision::Symbol; time_input = false)
    d = Ref(mlp_desc(model; time_input))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gbnde_create, libgbnde), Cint, (Ptr{Ptr{Cvoid}}, Ref{MlpDesc}, Cint, Cint),
                h, d, precision === :bf16 ? 1 : 0, 0))
    c = Ctx(h[], Int(ccall((:gbnde_nparams, libgbnde), Csize_t, (Ptr{Cvoid},), h[])))
    finalizer(x -> ccall((:gbnde_destroy, libgbnde), Cvoid, (Ptr{Cvoid},), x.h), c)
    c
end

const CTXS = IdDict{Any, Ctx}()
ctx_for(model, prec) = get!(() -> Ctx(model, prec), CTXS, (model, prec))

sensecode(s) = s isa BacksolveAdjoint ? 1 : s isa InterpolatingAdjoint ? 0 :
               (s isa QuadratureAdjoint || s isa GaussAdjoint) ? 2 :
               error("GB300 supports InterpolatingAdjoint, BacksolveAdjoint, QuadratureAdjoint and GaussAdjoint")

# ---- the differentiable solve -------------------------------------------------------------
"""
    gb300_solve(u0, p, ctx, tspan, saveat, abstol, reltol, sensealg, flags) -> Array (S, B, nsave)

`flags = GBNDE_FLAG_FP32_TIME` keeps t and dt in Float32 (the FP32 form with a Float32 tspan).
"""
const GBNDE_FLAG_FP32_TIME = Cint(1)
function gb300_solve(u0::AbstractMatrix{Float32}, p::AbstractVector{Float32}, ctx::Ctx, tspan,
                     saveat::Vector{Float64}, abstol, reltol, sensealg, flags = Cint(0))
    S, B = size(u0)
    check(ccall((:gbnde_set_params, libgbnde), Cint, (Ptr{Cvoid}, Ptr{Float32}, Csize_t),
                ctx.h, p, length(p)))
    out = Array{Float32}(undef, S, B, length(saveat))
    st = Stats()
    GC.@preserve saveat begin
        d = Ref(SolveDesc(tspan[1], tspan[2], abstol, reltol, 0, 0, 100000, pointer(saveat),
                          length(saveat), sensecode(sensealg), flags))
        check(ccall((:gbnde_forward, libgbnde), Cint,
                    (Ptr{Cvoid}, Ref{SolveDesc}, Cint, Cint, Ptr{Float32}, Ptr{Float32}, Ref{Stats}),
                    ctx.h, d, S, B, Matrix(u0), out, st))
    end
    out, st
end

function ChainRulesCore.rrule(::typeof(gb300_solve), u0, p, ctx, tspan, saveat, abstol, reltol,
                              sensealg, flags = Cint(0))
    out, st = gb300_solve(u0, p, ctx, tspan, saveat, abstol, reltol, sensealg, flags)
    function pullback(Δ)
        Δo = unthunk(Δ[1])
        du0 = similar(u0)
        dp = similar(p)
        bst = Stats()
        check(ccall((:gbnde_backward, libgbnde), Cint,
                    (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Ref{Stats}),
                    ctx.h, Array{Float32}(Δo), du0, dp, bst))
        (NoTangent(), du0, dp, NoTangent(), NoTangent(), NoTangent(), NoTangent(), NoTangent(),
         NoTangent(), NoTangent())
    end
    (out, st), pullback
end

# ---- NeuralODE on the GB300 path (src/neural_de.jl:47-61) --------------------------------
function (n::NeuralODE)(x, p, st, alg::GB300Tsit5)
    kw = Dict(n.kwargs)
    saveat = Float64.(collect(get(kw, :saveat, [n.tspan[2]])))
    ctx = ctx_for(n.model, alg.precision)
    sense = get(kw, :sensealg, InterpolatingAdjoint(; autojacvec = ZygoteVJP()))
    u0 = x isa AbstractVector ? reshape(x, :, 1) : x
    # a Float32 tspan keeps t and dt in Float32, as the reference's integrator does
    flags = (eltype(n.tspan) === Float32 && alg.precision === :fp32) ? GBNDE_FLAG_FP32_TIME : Cint(0)
    out, stats = gb300_solve(Float32.(u0), Float32.(collect(p)), ctx, Float64.(n.tspan), saveat,
                             get(kw, :abstol, 1e-6), get(kw, :reltol, 1e-3), sense, flags)
    prob = ODEProblem{false}((u, p, t) -> u, x, n.tspan, p)
    us = [x isa AbstractVector ? out[:, 1, i] : out[:, :, i] for i in axes(out, 3)]
    sol = SciMLBase.build_solution(prob, alg, saveat, us; retcode = RETCODES[stats.retcode + 1])
    sol, st
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

end # module
