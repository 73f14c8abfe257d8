# check_reference.jl -- pins the oracle (and the GB300 route) to the reference.
#
# Run where Julia and the reference's stack are installed (DiffEqFlux,
# OrdinaryDiffEq, SciMLSensitivity, Lux, ComponentArrays, Zygote, NPZ), from the
# repository root:
#
#     julia --project=<env with those packages> tests/golden/check_reference.jl [--gb300]
#
# For each fixture written by tests/golden/make_golden.py it rebuilds the same
# problem for the reference -- the flat parameter vector in the ComponentArray
# order, the same u0, save times and tolerances -- and runs the reference's own
# `NeuralODE` (src/neural_de.jl:47-61) with Tsit5 and both adjoints
# (InterpolatingAdjoint, the default; BacksolveAdjoint,
# test/BasicNeuralDE/neural_de_tests.jl:36). It prints the relative
# differences of the saved states, dL/du0 and dL/dp against the fixture's FP64
# oracle values, and the accepted/rejected step counts of the reference's
# forward solve against the oracle's. With --gb300 the same problems also run
# through DiffEqFluxGB300 (:fp32 form), so one session compares all three.
#
# ffjord.npz runs the reference's FFJORD (src/ffjord.jl:138-178) with the exact
# trace (st.monte_carlo = false, deterministic) and compares logpx and the
# gradients of -mean(logpx); multishoot.npz runs the reference's
# multiple_shoot (src/multiple_shooting.jl:36-94) with the SSE loss and
# compares the loss, the group predictions and dL/dp.
using DiffEqFlux, OrdinaryDiffEq, SciMLSensitivity, Lux, ComponentArrays, Zygote, NPZ, Random, LinearAlgebra,
      Statistics

const HERE = @__DIR__
const WITH_GB300 = "--gb300" in ARGS
if WITH_GB300
    include(joinpath(HERE, "..", "..", "diffeqflux.jl_gb300", "julia", "DiffEqFluxGB300.jl"))
    using .DiffEqFluxGB300
end

reldiff(a, b) = norm(vec(Float64.(a)) .- vec(Float64.(b))) / max(norm(vec(Float64.(b))), 1e-300)

function build(fx)
    dims = Int.(fx["dims"])
    layers = Any[]
    fx["cube"] == 1 && push!(layers, WrappedFunction(x -> x .^ 3))
    for l in 1:(length(dims) - 1)
        act = l < length(dims) - 1 ? tanh : identity
        push!(layers, Dense(dims[l] => dims[l + 1], act))
    end
    Chain(layers...)
end

function check(name; loss_kind)
    fx = npzread(joinpath(HERE, "$name.npz"))
    model = build(fx)
    ts = vec(fx["ts"])
    tspan = (Float32(ts[1]), Float32(ts[end]))
    u0 = Float32.(fx["u0"])
    ps0, st = Lux.setup(Random.default_rng(), model)
    ax = getaxes(ComponentArray(ps0))
    p = ComponentArray(Float32.(vec(fx["p"])), ax)   # same flat order as the fixture
    dL = fx["dLdu"]
    println("== $name: dims $(Int.(fx["dims"])), $(size(u0, 2)) trajectories, $(length(ts)) saves")
    for (label, sense, gu_ref, gp_ref) in (
            ("InterpolatingAdjoint", InterpolatingAdjoint(; autojacvec = ZygoteVJP()), fx["gu_interp"], fx["gp_interp"]),
            ("BacksolveAdjoint", BacksolveAdjoint(; autojacvec = ZygoteVJP()), fx["gu_back"], fx["gp_back"]))
        node = NeuralODE(model, tspan, Tsit5(); saveat = Float32.(ts), abstol = fx["abstol"],
                         reltol = fx["reltol"], sensealg = sense)
        sol, _ = node(u0, p, st)
        us = Array(sol)
        println("  reference forward: saves rel diff $(reldiff(us, fx["usave"])), ",
                "steps $(sol.stats.naccept) accepted / $(sol.stats.nreject) rejected ",
                "(oracle $(fx["naccept"]) / $(fx["nreject"]))")
        # the fixture's cotangent dL/dusave is linear in the saves: <dL, usave>
        # has exactly that cotangent
        gu, gp = Zygote.gradient((x, q) -> sum(Float64.(dL) .* Array(first(node(x, q, st)))), u0, p)
        println("  reference $label: dL/du0 rel diff $(reldiff(gu, gu_ref)), dL/dp rel diff $(reldiff(gp, gp_ref))")
        if WITH_GB300
            gnode = gb300(node, GB300Tsit5(:fp32))
            gsol, _ = gnode(u0, p, st)
            ggu, ggp = Zygote.gradient((x, q) -> sum(Float64.(dL) .* Array(first(gnode(x, q, st)))), u0, p)
            println("  GB300 fp32 $label: saves vs reference $(reldiff(Array(gsol), us)), ",
                    "dL/du0 $(reldiff(ggu, gu)), dL/dp $(reldiff(ggp, gp))")
        end
    end
end

check("spiral"; loss_kind = :sse)
check("batched"; loss_kind = :mse)

function check_ffjord()
    fx = npzread(joinpath(HERE, "ffjord.npz"))
    d, H = Int(fx["dims"][1]), Int(fx["dims"][2])
    nn = Chain(Dense(d => H, tanh), Dense(H => d))
    x = Float32.(fx["x"])
    ff = FFJORD(nn, (0.0f0, 1.0f0), (d,), Tsit5(); abstol = fx["abstol"], reltol = fx["reltol"])
    ps0, st = Lux.setup(Random.default_rng(), ff)
    st = (; st..., monte_carlo = false, regularize = false)
    p = ComponentArray(Float32.(vec(fx["p"])), getaxes(ComponentArray(ps0)))
    nll(q, xx) = -mean(first(first(ff(xx, q, st))))
    logpx = vec(first(first(ff(x, p, st))))
    gp, gx = Zygote.gradient(nll, p, x)
    println("== ffjord: d $d, $(size(x, 2)) samples, exact trace")
    println("  reference: logpx rel diff $(reldiff(logpx, fx["logpx"])), ",
            "dL/dp rel diff $(reldiff(gp, fx["gp"])), dL/dx rel diff $(reldiff(gx, fx["gx"]))")
    if WITH_GB300
        gff = gb300(ff, GB300Tsit5(:fp32))
        glogpx = vec(first(first(gff(x, p, st))))
        ggp = first(Zygote.gradient(q -> -mean(first(first(gff(x, q, st)))), p))
        println("  GB300 fp32: logpx vs reference $(reldiff(glogpx, logpx)), dL/dp $(reldiff(ggp, gp))")
    end
end

function check_multishoot()
    fx = npzread(joinpath(HERE, "multishoot.npz"))
    S, H = Int(fx["dims"][1]), Int(fx["dims"][2])
    nn = Chain(Dense(S => H, tanh), Dense(H => S))
    ps0, st = Lux.setup(Random.default_rng(), nn)
    p = ComponentArray(Float32.(vec(fx["p"])), getaxes(ComponentArray(ps0)))
    smodel = StatefulLuxLayer{true}(nn, nothing, st)
    data = Float32.(fx["data"])
    ts = Float32.(vec(fx["ts"]))
    prob = ODEProblem((u, q, t) -> smodel(u, q), data[:, 1], (ts[1], ts[end]), p)
    sse(u, uh) = sum(abs2, u .- uh)
    ms(q) = multiple_shoot(q, data, ts, prob, sse, Tsit5(), Int(fx["group_size"]);
                           continuity_term = fx["continuity_term"], abstol = fx["abstol"], reltol = fx["reltol"])
    loss, preds = ms(p)
    gp = first(Zygote.gradient(q -> first(ms(q)), p))
    println("== multishoot: state $S, $(size(data, 2)) points, group size $(Int(fx["group_size"]))")
    println("  reference: loss rel diff $(abs(loss - fx["loss"]) / abs(fx["loss"])), ",
            "predictions rel diff $(reldiff(reduce(hcat, Array.(preds)), fx["preds"])), ",
            "dL/dp rel diff $(reldiff(gp, fx["gp"]))")
end

check_ffjord()
check_multishoot()
