"""BF16 tensor-core form (split-BF16 tcgen05 GEMMs, FP32 state, FP64 control)
against the FP64 oracle and against the plain FP32 form, through the C ABI.

Tolerances (relative):
  * saved states vs the oracle replaying the kernel's accepted steps: 2e-5
  * loss and gradient vs the FP64 oracle (the benchmark's validity bar): 1e-3
  * saved states vs the FP32 form at the headline batch: 1e-4
"""
import numpy as np
import pytest

from conftest import gpu_available
from test_gpu_neural_ode import _oracle, _rel, _setup

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]


def _node(model, ts, prec, abstol, reltol, sensealg=None):
    import gbnde
    return gbnde.NeuralODE(model, (0.0, float(ts[-1])), gbnde.Tsit5(prec), saveat=ts, abstol=abstol,
                           reltol=reltol, sensealg=sensealg)


@pytest.mark.parametrize("B", [128, 300])
def test_bf16_forward_and_gradient_vs_oracle(B):
    from oracle import tsit5 as ots
    S, H = 64, 256
    model, p, rng = _setup([S, H, H, S], ["tanh", "tanh", "identity"], False, B, 2, bias=0.02)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, 20)
    node = _node(model, ts, "bf16", 1e-7, 1e-5)
    s = node.solver
    s.set_params(p)
    us, st = s.forward(u0, node.desc())
    assert st.retcode == 0
    steps = s.forward_steps()
    rhs = _oracle(model, p)
    ous, fwd = ots.solve_forward(rhs, u0.astype(np.float64), 0.0, 1.0, ts, 1e-7, 1e-5, steps=steps)
    assert _rel(us, ous) < 2e-5
    # loss / gradient against the free-running FP64 oracle
    ous2, fwd2 = ots.solve_forward(_oracle(model, p), u0.astype(np.float64), 0.0, 1.0, ts, 1e-7, 1e-5)
    tgt = np.zeros_like(ous2)
    L64 = np.mean((ous2 - tgt) ** 2)
    L = np.mean((us.astype(np.float64) - tgt) ** 2)
    assert abs(L - L64) / L64 < 1e-3
    g = (2.0 * (us.astype(np.float64) - tgt) / us.size).astype(np.float32)
    du0, dp, sta = s.backward(g)
    assert sta.retcode_adj == 0
    gu, gp, _ = ots.adjoint_interpolating(_oracle(model, p), fwd2, ts, 2.0 * (ous2 - tgt) / ous2.size,
                                          0.0, 1e-7, 1e-5)
    assert _rel(du0, gu) < 1e-3
    assert _rel(dp, gp) < 1e-3
    # the split products keep the step count near the FP64 controller's
    assert st.naccept + st.nreject <= 3 * (fwd2.naccept + fwd2.nreject) + 4


def test_bf16_matches_fp32_form_at_headline_batch():
    S, H, B = 64, 256, 16384
    model, p, rng = _setup([S, H, H, S], ["tanh", "tanh", "identity"], False, B, 1, bias=0.0)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, 20)
    out = {}
    for prec in ("fp32", "bf16"):
        node = _node(model, ts, prec, 1e-7, 1e-5)
        s = node.solver
        s.set_params(p)
        us, st = s.forward(u0, node.desc())
        assert st.retcode == 0
        g = np.ones_like(us) / us.size
        du0, dp, sta = s.backward(g)
        assert sta.retcode_adj == 0
        # the tensor-core adjoint reuses the previous activations at every
        # interval start after the first (19 save intervals -> 18) and at stage
        # 7 of every attempted step
        want = (len(ts) - 2) + sta.naccept_adj + sta.nreject_adj if prec == "bf16" else 0
        assert sta.nf_adj_vjp == want, (sta.nf_adj_vjp, want)
        out[prec] = (us, du0, dp, st)
    assert _rel(out["bf16"][0], out["fp32"][0].astype(np.float64)) < 1e-4
    assert _rel(out["bf16"][1], out["fp32"][1].astype(np.float64)) < 1e-3
    assert _rel(out["bf16"][2], out["fp32"][2].astype(np.float64)) < 1e-3


@pytest.mark.parametrize("S,H,cube", [(2, 50, True), (32, 128, False), (16, 64, False)])
def test_bf16_small_shapes(S, H, cube):
    """Padded shapes: state < 64, hidden not a multiple of 64, cube prefix."""
    from oracle import tsit5 as ots
    B = 200
    model, p, rng = _setup([S, H, S], ["tanh", "identity"], cube, B, 3)
    u0 = rng.standard_normal((S, B)).astype(np.float32) * (0.5 if cube else 1.0)
    ts = np.linspace(0.0, 1.0, 8)
    node = _node(model, ts, "bf16", 1e-6, 1e-4)
    s = node.solver
    s.set_params(p)
    us, st = s.forward(u0, node.desc())
    assert st.retcode == 0
    ous, _ = ots.solve_forward(_oracle(model, p), u0.astype(np.float64), 0.0, 1.0, ts, 1e-6, 1e-4,
                               steps=s.forward_steps())
    assert _rel(us, ous) < 2e-5


@pytest.mark.parametrize("S,H,cube,B", [(2, 50, True, 200), (32, 128, False, 300), (48, 96, False, 130)])
def test_bf16_small_shapes_gradient(S, H, cube, B):
    """Tensor-core adjoint at padded shapes (state below 64 and not a multiple
    of 32, hidden widths not multiples of 64, a partial last tile), against
    the FP64 oracle's InterpolatingAdjoint."""
    from oracle import tsit5 as ots
    model, p, rng = _setup([S, H, S], ["tanh", "identity"], cube, B, 5)
    u0 = rng.standard_normal((S, B)).astype(np.float32) * (0.5 if cube else 1.0)
    ts = np.linspace(0.0, 1.0, 6)
    node = _node(model, ts, "bf16", 1e-6, 1e-4)
    s = node.solver
    s.set_params(p)
    us, st = s.forward(u0, node.desc())
    assert st.retcode == 0
    rhs = _oracle(model, p)
    ous, fwd = ots.solve_forward(rhs, u0.astype(np.float64), 0.0, 1.0, ts, 1e-6, 1e-4)
    g = (2.0 * us.astype(np.float64) / us.size).astype(np.float32)
    du0, dp, sta = s.backward(g)
    assert sta.retcode_adj == 0
    gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, ts, 2.0 * ous / ous.size, 0.0, 1e-6, 1e-4)
    assert _rel(du0, gu) < 1e-3
    assert _rel(dp, gp) < 1e-3


@pytest.mark.parametrize("case", ["tanh_output", "backsolve"])
def test_bf16_forward_with_fp32_adjoint(case):
    """Models the tensor-core adjoint does not cover (a non-identity output
    layer) and BacksolveAdjoint run the BF16 forward with the FP32 adjoint:
    it must not read the forward's tile-layout stage storage, and the
    gradient still matches the FP64 oracle."""
    import gbnde
    from oracle import tsit5 as ots
    S, H, B = 16, 64, 256
    acts = ["tanh", "tanh"] if case == "tanh_output" else ["tanh", "identity"]
    model, p, rng = _setup([S, H, S], acts, False, B, 7)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, 6)
    sense = gbnde.BacksolveAdjoint() if case == "backsolve" else gbnde.InterpolatingAdjoint()
    node = _node(model, ts, "bf16", 1e-6, 1e-4, sensealg=sense)
    s = node.solver
    s.set_params(p)
    us, st = s.forward(u0, node.desc())
    assert st.retcode == 0
    rhs = _oracle(model, p)
    ous, fwd = ots.solve_forward(rhs, u0.astype(np.float64), 0.0, 1.0, ts, 1e-6, 1e-4)
    g = (2.0 * us.astype(np.float64) / us.size).astype(np.float32)
    du0, dp, sta = s.backward(g)
    assert sta.retcode_adj == 0
    dl = 2.0 * ous / ous.size
    if case == "backsolve":
        gu, gp, _ = ots.adjoint_backsolve(rhs, ous, ts, dl, 0.0, 1e-6, 1e-4)
    else:
        gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, ts, dl, 0.0, 1e-6, 1e-4)
    assert _rel(du0, gu) < 2e-3
    assert _rel(dp, gp) < 2e-3


def test_bf16_batch_above_one_tile_per_sm():
    """More 128-trajectory tiles than SMs: the tensor-core forward runs several
    tiles per CTA, and the gradient (which then takes the FP32 adjoint) must
    match the FP32 form as at smaller batches."""
    import torch
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    S, H, B = 16, 64, 128 * (nsm + 8)
    model, p, rng = _setup([S, H, H, S], ["tanh", "tanh", "identity"], False, B, 4, bias=0.0)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, 8)
    out = {}
    for prec in ("fp32", "bf16"):
        node = _node(model, ts, prec, 1e-7, 1e-5)
        s = node.solver
        s.set_params(p)
        us, st = s.forward(u0, node.desc())
        assert st.retcode == 0
        g = np.ones_like(us) / us.size
        du0, dp, sta = s.backward(g)
        assert sta.retcode_adj == 0
        out[prec] = (us, du0, dp)
    assert _rel(out["bf16"][0], out["fp32"][0].astype(np.float64)) < 1e-4
    assert _rel(out["bf16"][1], out["fp32"][1].astype(np.float64)) < 1e-3
    assert _rel(out["bf16"][2], out["fp32"][2].astype(np.float64)) < 1e-3


@pytest.mark.parametrize("nsave", [4, 20])
def test_bf16_checkpoint_replay_matches_dense_storage(nsave):
    """O(checkpoints) memory in the BF16 form: with the dense stage storage
    capped (gbnde_set_stage_memory), the tensor-core adjoint replays every
    save interval's forward steps on the tensor cores from its checkpoint
    (state and compensation) -- bit-identical to the forward -- so its
    gradient matches the dense-storage gradient to 1e-5 (to the last bit in
    practice), and gbnde_stats.adj_path reports the recompute path."""
    import ctypes as C

    from gbnde import _lib
    S, H, B = 64, 256, 300
    model, p, rng = _setup([S, H, H, S], ["tanh", "tanh", "identity"], False, B, 4, bias=0.02)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, nsave)
    node = _node(model, ts, "bf16", 1e-7, 1e-5)
    s = node.solver
    s.set_params(p)
    us, st = s.forward(u0, node.desc())
    g = (0.1 * rng.standard_normal(us.shape)).astype(np.float32)
    du0, dp, sta = s.backward(g)
    assert sta.adj_path == _lib.PATH_TC and sta.nf_recompute == 0
    _lib.check(s.lib.gbnde_set_stage_memory(s.h, C.c_size_t(1)))
    us2, st2 = s.forward(u0, node.desc())
    assert np.array_equal(us2, us) and st2.naccept == st.naccept
    du0r, dpr, star = s.backward(g)
    assert star.retcode_adj == 0
    assert star.adj_path == _lib.PATH_TC_RECOMPUTE
    # every interval replays its steps: at least 6 evaluations per forward step, plus its first k1
    assert star.nf_recompute >= 6 * st.naccept + 1
    assert _rel(du0r, du0) < 1e-5 and _rel(dpr, dp) < 1e-5
    assert star.naccept_adj == sta.naccept_adj
    _lib.check(s.lib.gbnde_set_stage_memory(s.h, C.c_size_t(0)))
    us3, _ = s.forward(u0, node.desc())
    _, _, sta3 = s.backward(g)
    assert sta3.adj_path == _lib.PATH_TC
