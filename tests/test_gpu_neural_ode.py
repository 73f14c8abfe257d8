"""GPU parity of the NeuralODE forward solve and adjoint gradient (FP32 form)
against the FP64 CPU oracle, through the C ABI.

Mirrors the reference's hot-path tests (test/BasicNeuralDE/neural_de_tests.jl:7-59:
Chain(Dense(2=>50,tanh), Dense(50=>2)), u0 = [2,0] and a 2x3 batch, default /
tight tolerances, BacksolveAdjoint, saveat range) but asserts values, not
only non-zero gradients.

Tolerances (relative, FP32 kernel vs FP64 oracle):
  * replayed steps (oracle takes the GPU's accepted steps): 2e-5 on saved states
  * gradients (both adjoints adaptive, FP32 vs FP64 rounding in the controller): 2e-4
"""
import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _setup(dims, acts, cube, B, seed, bias=0.05):
    import gbnde
    rng = np.random.default_rng(seed)
    layers = [gbnde.cube()] if cube else []
    layers += [gbnde.Dense(dims[i], dims[i + 1], acts[i]) for i in range(len(acts))]
    model = gbnde.Chain(*layers)
    p = model.init_params(rng)
    off = 0
    for i in range(len(acts)):
        off += dims[i] * dims[i + 1]
        p[off:off + dims[i + 1]] = bias * rng.standard_normal(dims[i + 1])
        off += dims[i + 1]
    return model, p, rng


def _oracle(model, p):
    from oracle import mlp as omlp
    om = omlp.MLP(model.dims, model.acts, cube_input=model.cube_input)
    return omlp.MLPRHS(om, np.asarray(p, np.float64))


def _run_case(model, p, u0, tspan, ts, abstol, reltol, sensealg, precision="fp32"):
    import gbnde
    from oracle import tsit5 as ots
    node = gbnde.NeuralODE(model, tspan, gbnde.Tsit5(precision), saveat=ts, abstol=abstol,
                           reltol=reltol, sensealg=sensealg)
    solver = node.solver
    solver.set_params(p)
    usave, st = solver.forward(u0, node.desc())
    assert st.retcode == 0
    rhs = _oracle(model, p)
    steps = solver.forward_steps()
    assert len(steps) == st.naccept
    # replayed steps: isolates FP32 rounding of the kernel
    ous, fwd = ots.solve_forward(rhs, u0.astype(np.float64), tspan[0], tspan[1], ts, abstol, reltol,
                                 steps=steps)
    # free-running oracle: same controller, FP64 everywhere
    ous2, fwd2 = ots.solve_forward(_oracle(model, p), u0.astype(np.float64), tspan[0], tspan[1], ts,
                                   abstol, reltol)
    rng = np.random.default_rng(7)
    target = ous + 0.1 * rng.standard_normal(ous.shape)
    g = 2.0 * (usave.astype(np.float64) - target)
    du0, dp, sta = solver.backward(g.astype(np.float32))
    assert sta.retcode_adj == 0
    if sensealg.code == 0:
        gu, gp, bint = ots.adjoint_interpolating(rhs, fwd, ts, g, tspan[0], abstol, reltol)
    else:
        gu, gp, bint = ots.adjoint_backsolve(rhs, ous, ts, g, tspan[0], abstol, reltol)
    return dict(usave=usave, ous=ous, ous2=ous2, st=st, fwd2=fwd2, du0=du0, dp=dp, gu=gu, gp=gp,
                sta=sta, bint=bint)


def test_spiral_config_forward_and_gradient():
    """cube -> Dense(2,50,tanh) -> Dense(50,2), u0=[2,0], tspan (0,1.5), 30 saveat,
    abstol 1e-7 / reltol 1e-5 (docs/src/examples/neural_ode.md:19-36)."""
    import gbnde
    model, p, _ = _setup([2, 50, 2], ["tanh", "identity"], True, 1, 0)
    u0 = np.array([[2.0], [0.0]], np.float32)
    ts = np.linspace(0.0, 1.5, 30)
    r = _run_case(model, p, u0, (0.0, 1.5), ts, 1e-7, 1e-5, gbnde.InterpolatingAdjoint())
    assert _rel(r["usave"], r["ous"]) < 2e-5
    # free-running FP64 oracle: at abstol 1e-7 the FP32 rounding floor of the
    # embedded error estimate makes the FP32 controller take smaller steps, so
    # only the solution (not the step count) is compared here
    assert _rel(r["usave"], r["ous2"]) < 1e-4
    assert _rel(r["du0"], r["gu"]) < 2e-4
    assert _rel(r["dp"], r["gp"]) < 2e-4


@pytest.mark.parametrize("B", [1, 50])
@pytest.mark.parametrize("tol", [1e-4, 1e-7])
def test_controller_replays_trace(B, tol):
    """The PI controller, the initial step and the clipping to t1 act exactly as
    restated in the oracle, given the error estimates the kernel measured: the
    kernel's trace of attempted steps (t, h, EEst, accepted) is replayed through
    the controller formula and every next step size must agree to 1e-12.
    (The estimates themselves are compared only through the solution: at these
    tolerances the FP32 rounding floor of EEst differs from the FP64 value.)"""
    import gbnde
    from oracle import tableau as T
    model, p, rng = _setup([2, 50, 2], ["tanh", "identity"], True, B, 0)
    u0 = (rng.standard_normal((2, B)) + np.array([[2.0], [0.0]])).astype(np.float32)
    ts = np.linspace(0.0, 1.5, 30)
    node = gbnde.NeuralODE(model, (0.0, 1.5), gbnde.Tsit5(), saveat=ts, abstol=tol, reltol=tol)
    s = node.solver
    s.set_params(p)
    us, st = s.forward(u0, node.desc())
    tr = s.forward_trace()
    assert len(tr) == st.naccept + st.nreject
    assert st.nf == 2 + 6 * len(tr)
    t1, qold = 1.5, T.QOLDINIT
    for i in range(len(tr) - 1):
        t, h, e, acc = tr[i]
        tn, hn = tr[i + 1][:2]
        if e == 0.0:
            q, q11 = 1.0 / T.QMAX, 0.0
        else:
            q11 = e ** T.BETA1
            q = max(1.0 / T.QMAX, min(1.0 / T.QMIN, q11 / qold ** T.BETA2 / T.GAMMA))
        if acc:
            assert tn == (t1 if t + h >= t1 else t + h) or abs(tn - (t + h)) <= 1e-15
            if T.QSTEADY_MIN <= q <= T.QSTEADY_MAX:
                q = 1.0
            qold = max(e, T.QOLDINIT)
            dt = min(abs(h) / q, 1.5)
        else:
            assert tn == t
            dt = abs(h) / min(1.0 / T.QMIN, q11 / T.GAMMA)
        assert abs(hn - min(dt, t1 - tn)) <= 1e-12 * hn
    assert tr[-1][3] and tr[-1][0] + tr[-1][1] >= 1.5 - 1e-12


@pytest.mark.parametrize("sense", ["interpolating", "backsolve"])
@pytest.mark.parametrize("B", [3, 100, 257])
def test_batched_tanh_mlp(sense, B):
    """2-hidden-layer tanh MLP, ragged batch sizes (not multiples of the tile)."""
    import gbnde
    S, H = 16, 64
    model, p, rng = _setup([S, H, H, S], ["tanh", "tanh", "identity"], False, B, 1)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, 11)
    sa = gbnde.InterpolatingAdjoint() if sense == "interpolating" else gbnde.BacksolveAdjoint()
    r = _run_case(model, p, u0, (0.0, 1.0), ts, 1e-6, 1e-4, sa)
    assert _rel(r["usave"], r["ous"]) < 2e-5
    assert _rel(r["du0"], r["gu"]) < 5e-4
    assert _rel(r["dp"], r["gp"]) < 5e-4


def test_config2_shape_small_batch():
    """State 64, MLP 64->256->256->64 tanh, 20 saveat on (0,1), abstol 1e-7 reltol 1e-5
    (the batched headline configuration at a batch the FP64 oracle finishes quickly)."""
    import gbnde
    S, H, B = 64, 256, 192
    model, p, rng = _setup([S, H, H, S], ["tanh", "tanh", "identity"], False, B, 2, bias=0.0)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, 20)
    r = _run_case(model, p, u0, (0.0, 1.0), ts, 1e-7, 1e-5, gbnde.InterpolatingAdjoint())
    assert _rel(r["usave"], r["ous"]) < 2e-5
    assert _rel(r["du0"], r["gu"]) < 2e-4
    assert _rel(r["dp"], r["gp"]) < 2e-4


def test_deterministic_bitwise():
    import gbnde
    S, H, B = 16, 64, 300
    model, p, rng = _setup([S, H, H, S], ["tanh", "tanh", "identity"], False, B, 3)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5("fp32"), saveat=np.linspace(0, 1, 5),
                           abstol=1e-6, reltol=1e-4)
    s = node.solver
    s.set_params(p)
    a, _ = s.forward(u0, node.desc())
    g = np.ones_like(a)
    da, pa, _ = s.backward(g)
    b, _ = s.forward(u0, node.desc())
    db, pb, _ = s.backward(g)
    assert np.array_equal(a, b) and np.array_equal(da, db) and np.array_equal(pa, pb)


def test_retcodes_maxiters_and_unstable():
    import gbnde
    S, H, B = 4, 16, 8
    model, p, rng = _setup([S, H, S], ["tanh", "identity"], False, B, 4)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5(), saveat=[0.0, 1.0], abstol=1e-9,
                           reltol=1e-9, maxiters=3)
    s = node.solver
    s.set_params(p)
    _, st = s.forward(u0, node.desc())
    assert st.retcode == 1  # MaxIters
    u0[0, 0] = np.nan
    node2 = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5(), saveat=[0.0, 1.0])
    s2 = node2.solver
    s2.set_params(p)
    _, st2 = s2.forward(u0, node2.desc())
    assert st2.retcode == 3  # Unstable
    with pytest.raises(gbnde.GbndeError):
        s2.backward(np.ones((S, B, 2), np.float32))


def test_torch_autograd_bridge():
    import torch

    import gbnde
    S, H, B = 8, 32, 64
    model, p, rng = _setup([S, H, S], ["tanh", "identity"], False, B, 5)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5(), saveat=np.linspace(0, 1, 4),
                           abstol=1e-6, reltol=1e-4)
    x = torch.tensor(u0, device="cuda", requires_grad=True)
    pt = torch.tensor(p, device="cuda", requires_grad=True)
    sol, _ = node(x, pt, {})
    loss = (sol.array() ** 2).sum()
    loss.backward()
    s = node.solver
    s.set_params(p)
    us, _ = s.forward(u0, node.desc())
    du0, dp, _ = s.backward(2.0 * us)
    assert np.allclose(x.grad.cpu().numpy(), du0, rtol=1e-5, atol=1e-6)
    assert np.allclose(pt.grad.cpu().numpy(), dp, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
@pytest.mark.parametrize("marker", ["GaussAdjoint", "QuadratureAdjoint"])
def test_quadrature_adjoint_against_oracle(prec, marker):
    """QuadratureAdjoint / GaussAdjoint: lam-only backward solve plus 4-point
    Gauss-Legendre quadrature of lam^T df/dp over every accepted adjoint step,
    against the FP64 oracle's restatement (itself checked against central
    finite differences) and against the InterpolatingAdjoint gradient."""
    import gbnde
    from oracle import tsit5 as ots
    S, H, B = 8, 32, 96
    model, p, rng = _setup([S, H, H, S], ["tanh", "tanh", "identity"], False, B, 13)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, 6)
    tol = 1e-6
    out = {}
    for name, sense in (("q", getattr(gbnde, marker)()), ("i", gbnde.InterpolatingAdjoint())):
        node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5(prec), saveat=ts, abstol=tol, reltol=tol,
                               sensealg=sense)
        s = node.solver
        s.set_params(p)
        us, st = s.forward(u0, node.desc())
        assert st.retcode == 0
        du0, dp, sta = s.backward(2.0 * us / us.size)
        assert sta.retcode_adj == 0
        out[name] = (us, du0, dp)
    rhs = _oracle(model, p)
    ous, fwd = ots.solve_forward(rhs, u0.astype(np.float64), 0.0, 1.0, ts, tol, tol)
    gu, gp, _ = ots.adjoint_gauss(rhs, fwd, ts, 2.0 * ous / ous.size, 0.0, tol, tol)
    tolg = 1e-4 if prec == "fp32" else 1e-3
    assert _rel(out["q"][1], gu) < tolg
    assert _rel(out["q"][2], gp) < tolg
    assert _rel(out["q"][2], out["i"][2].astype(np.float64)) < 1e-3


@pytest.mark.parametrize("B", [1, 64])
def test_float32_time_mode(B):
    """GBNDE_FLAG_FP32_TIME (a Float32 tspan, as the reference's integrator keeps
    t and dt in Float32): every accepted step starts at a Float32 time with a
    Float32 step; states and gradients match the oracle run in the same mode
    (replayed steps 2e-5, adaptive adjoint 2e-4)."""
    import gbnde
    from oracle import tsit5 as ots
    model, p, rng = _setup([2, 50, 2], ["tanh", "identity"], True, B, 3)
    u0 = np.vstack([np.full((1, B), 2.0), 0.1 * rng.standard_normal((1, B))]).astype(np.float32)
    tspan = (np.float32(0.0), np.float32(1.5))
    ts = np.linspace(np.float32(0.0), np.float32(1.5), 30, dtype=np.float32)
    node = gbnde.NeuralODE(model, tspan, gbnde.Tsit5("fp32"), saveat=ts, abstol=1e-7, reltol=1e-5)
    assert node.float32_time
    s = node.solver
    s.set_params(p)
    us, st = s.forward(u0, node.desc())
    assert st.retcode == 0
    steps = s.forward_steps()
    assert len(steps) == st.naccept
    for tn, h in steps:
        assert float(np.float32(tn)) == tn and float(np.float32(h)) == abs(h), (tn, h)
    rhs = _oracle(model, p)
    ous, fwd = ots.solve_forward(rhs, u0.astype(np.float64), 0.0, 1.5, ts.astype(np.float64), 1e-7, 1e-5,
                                 steps=steps, time_f32=True)
    assert _rel(us, ous) < 2e-5
    g = (2.0 * (us.astype(np.float64) - 0.5 * ous)).astype(np.float32)
    du0, dp, sb = s.backward(g)
    assert sb.retcode_adj == 0
    gu, gp, integ = ots.adjoint_interpolating(rhs, fwd, ts.astype(np.float64), g.astype(np.float64), 0.0,
                                              1e-7, 1e-5, time_f32=True)
    for tn, h in integ.steps:
        assert float(np.float32(tn)) == tn
    assert _rel(du0, gu) < 2e-4
    assert _rel(dp, gp) < 2e-4
    # without the flag the same problem runs FP64 time
    node64 = gbnde.NeuralODE(model, (0.0, 1.5), gbnde.Tsit5("fp32"), saveat=ts, abstol=1e-7, reltol=1e-5)
    assert not node64.float32_time
    with pytest.raises(ValueError):
        gbnde.NeuralODE(model, tspan, gbnde.Tsit5("bf16"), saveat=ts, float32_time=True)


def test_barrier_wait_runs_out_and_reports():
    """Failure detection without a GPU fault: a grid barrier whose other CTA
    never arrives gives up after its limit and records the timeout; with both
    CTAs present it passes at once; the device stays usable afterwards."""
    import ctypes as C

    import gbnde
    from gbnde import _lib
    lib = gbnde.load(build_if_missing=True)
    t, w = C.c_int(-1), C.c_double(-1.0)
    _lib.check(lib.gbnde_barrier_selftest(-1, 50.0, C.byref(t), C.byref(w)))
    assert t.value == 0 and w.value < 50.0, (t.value, w.value)
    _lib.check(lib.gbnde_barrier_selftest(1, 50.0, C.byref(t), C.byref(w)))
    assert t.value == 1 and 45.0 <= w.value < 1000.0, (t.value, w.value)
    # a solve on the same device afterwards
    model, p, rng = _setup([2, 16, 2], ["tanh", "identity"], False, 4, 0)
    node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5("fp32"), saveat=[0.0, 1.0])
    node.solver.set_params(p)
    _, st = node.solver.forward(rng.standard_normal((2, 4)).astype(np.float32), node.desc())
    assert st.retcode == 0


@pytest.mark.parametrize("device", ["cpu", "cuda"])
def test_save_everystep_states_and_gradient(device):
    """No saveat: the reference saves every accepted step (save_everystep
    defaults to true, src/neural_de.jl:55-58 with the kwargs of
    test/BasicNeuralDE/neural_de_tests.jl:27-42). sol.t are t0 and every step
    end; the states are the oracle's at those times (replaying the steps), and
    the gradient of a loss of all of them matches the oracle's adjoint with
    those save points."""
    import torch

    import gbnde
    from oracle import tsit5 as ots
    model, p, rng = _setup([3, 16, 3], ["tanh", "identity"], False, 5, 9)
    node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5(), abstol=1e-6, reltol=1e-4)
    assert node.save_everystep
    dev = torch.device(device, 0) if device == "cuda" else torch.device("cpu")
    u0 = rng.standard_normal((3, 5)).astype(np.float32)
    x = torch.tensor(u0, device=dev, requires_grad=True)
    pt = torch.tensor(p, device=dev, requires_grad=True)
    sol, _ = node(x, pt, None)
    steps = node.solver.forward_steps()
    assert sol.t[0] == 0.0 and sol.t[-1] == 1.0 and len(sol.t) == len(steps) + 1
    assert all(abs(sol.t[k + 1] - (steps[k][0] + steps[k][1])) < 1e-12 for k in range(len(steps)))
    arr = sol.array()
    w = torch.tensor(rng.standard_normal(tuple(arr.shape)).astype(np.float32), device=dev)
    (arr * w).sum().backward()
    rhs = _oracle(model, p)
    ous, fwd = ots.solve_forward(rhs, u0.astype(np.float64), 0.0, 1.0, sol.t, 1e-6, 1e-4, steps=steps)
    assert _rel(arr.detach().cpu().numpy(), ous) < 2e-5
    gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, sol.t, w.cpu().numpy().astype(np.float64), 0.0, 1e-6, 1e-4)
    assert _rel(x.grad.cpu().numpy(), gu) < 2e-4
    assert _rel(pt.grad.cpu().numpy(), gp) < 2e-4


def test_c_abi_rejects_malformed_calls_before_any_launch():
    """Argument checks of the C entry points (the host side of the boundary;
    each call returns its error code before anything reaches the device):
    empty batch, t1 == t0, save times outside tspan or out of order, bad
    tolerances, a state size that does not match the model, unknown sensealg
    and flags, a backward before any forward, FFJORD's regularised form
    without noise, malformed multiple-shooting segments and reading saves
    before a multiple-shooting forward."""
    import ctypes as C

    import gbnde
    from gbnde import _lib as L
    S, H = 4, 8
    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, S))
    s = gbnde.Solver(model, "fp32", 0)
    s.set_params(model.init_params(np.random.default_rng(0)))
    lib, h = s.lib, s.h
    u0 = np.zeros((2, S), np.float32)
    us = np.zeros((4, 2, S), np.float32)
    st = L.Stats()

    def fwd(desc, S_=S, B=2):
        return lib.gbnde_forward(h, C.byref(desc), S_, B, u0.ctypes.data, us.ctypes.data, C.byref(st))

    D = gbnde.Solver.solve_desc
    assert fwd(D(0.0, 1.0, [0.0, 1.0], 1e-6, 1e-6), B=0) == L.ERR_INVALID
    assert fwd(D(0.0, 0.0, [0.0], 1e-6, 1e-6)) == L.ERR_INVALID
    assert fwd(D(0.0, 1.0, [0.0, 1.5], 1e-6, 1e-6)) == L.ERR_INVALID
    assert fwd(D(0.0, 1.0, [0.5, 0.2], 1e-6, 1e-6)) == L.ERR_INVALID
    assert fwd(D(0.0, 1.0, [1.0], 0.0, 1e-6)) == L.ERR_INVALID
    assert fwd(D(0.0, 1.0, [1.0], 1e-6, 1e-6), S_=S + 1) == L.ERR_INVALID
    assert fwd(D(0.0, 1.0, [1.0], 1e-6, 1e-6, sensealg=7)) == L.ERR_INVALID
    assert fwd(D(0.0, 1.0, [1.0], 1e-6, 1e-6, flags=0x100)) == L.ERR_INVALID
    dl = np.zeros((1, 2, S), np.float32)
    du0 = np.zeros((2, S), np.float32)
    dp = np.zeros(s.nparams, np.float32)
    assert lib.gbnde_backward(h, dl.ctypes.data, du0.ctypes.data, dp.ctypes.data, C.byref(st)) == L.ERR_STATE
    x = np.zeros((2, S), np.float32)
    lp = np.zeros(2, np.float32)
    desc = D(0.0, 1.0, [1.0], 1e-6, 1e-6)
    assert lib.gbnde_ffjord_forward_reg(h, C.byref(desc), S, 2, x.ctypes.data, None, 0, lp.ctypes.data, None,
                                        None, None, C.byref(st)) == L.ERR_INVALID
    seg = (L.Segment * 1)()
    seg[0].t0, seg[0].t1, seg[0].save_off, seg[0].nsave = 1.0, 0.0, 0, 1
    sv = np.array([0.5])
    ret = np.zeros(1, np.int32)
    assert lib.gbnde_multishoot_forward(h, S, 1, seg, sv.ctypes.data_as(C.POINTER(C.c_double)), 1,
                                        u0.ctypes.data, 1e-6, 1e-6, 1000, None,
                                        ret.ctypes.data_as(C.POINTER(C.c_int)), C.byref(st)) == L.ERR_INVALID
    assert lib.gbnde_multishoot_saves(h, us.ctypes.data) == L.ERR_STATE
    # a well-formed call still runs after the rejected ones
    assert fwd(D(0.0, 1.0, [0.0, 1.0], 1e-6, 1e-6)) == 0 and st.retcode == 0
    s.close()
