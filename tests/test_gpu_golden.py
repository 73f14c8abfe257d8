"""Both GPU forms against the committed golden fixtures (tests/golden/), through
the C ABI. linear.npz is a known answer (exact matrix exponential).

Tolerances (relative): FP32 form saved states 1e-4, gradients 5e-4;
BF16 form saved states 1e-4, gradients 1e-3 (the benchmark's validity bar)."""
import os

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def _node(g, prec, sense):
    import gbnde
    dims = [int(d) for d in g["dims"]]
    acts = ["tanh"] * (len(dims) - 2) + ["identity"]
    layers = [gbnde.cube()] if int(g["cube"]) else []
    layers += [gbnde.Dense(dims[i], dims[i + 1], acts[i]) for i in range(len(acts))]
    sa = gbnde.InterpolatingAdjoint() if sense == "interp" else gbnde.BacksolveAdjoint()
    node = gbnde.NeuralODE(gbnde.Chain(*layers), (0.0, float(g["ts"][-1])), gbnde.Tsit5(prec),
                           saveat=g["ts"], abstol=float(g["abstol"]), reltol=float(g["reltol"]),
                           sensealg=sa)
    node.solver.set_params(g["p"])
    return node


@pytest.mark.parametrize("prec,tol", [("fp32", 2e-6), ("bf16", 2e-5)])
def test_linear_known_answer(prec, tol):
    g = dict(np.load(os.path.join(GOLDEN, "linear.npz")))
    node = _node(g, prec, "interp")
    us, st = node.solver.forward(g["u0"].astype(np.float32), node.desc())
    assert st.retcode == 0
    assert _rel(us, g["exact"]) < tol


@pytest.mark.parametrize("name", ["spiral.npz", "batched.npz"])
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
@pytest.mark.parametrize("sense", ["interp", "back"])
def test_fixture_forward_and_gradient(name, prec, sense):
    g = dict(np.load(os.path.join(GOLDEN, name)))
    node = _node(g, prec, sense)
    us, st = node.solver.forward(g["u0"].astype(np.float32), node.desc())
    assert st.retcode == 0
    assert _rel(us, g["usave"]) < 1e-4
    du0, dp, sta = node.solver.backward(g["dLdu"].astype(np.float32))
    assert sta.retcode_adj == 0
    key = "interp" if sense == "interp" else "back"
    gtol = 5e-4 if prec == "fp32" else 1e-3
    assert _rel(du0, g["gu_" + key]) < gtol
    assert _rel(dp, g["gp_" + key]) < gtol


def test_ffjord_fixture_fp32():
    """ffjord.npz (exact trace, no time input): logpx and z(t1) 1e-4 relative
    to their max, and the gradients of -mean(logpx) in p and x 5e-4 (the
    fixture's oracle adjoint agrees with central differences to 1e-5)."""
    import gbnde
    g = dict(np.load(os.path.join(GOLDEN, "ffjord.npz")))
    d, H = int(g["dims"][0]), int(g["dims"][1])
    model = gbnde.Chain(gbnde.Dense(d, H, "tanh"), gbnde.Dense(H, d))
    fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5(), abstol=float(g["abstol"]),
                      reltol=float(g["reltol"]))
    B = g["x"].shape[1]
    logpx, zT, st = fj.forward_np(g["x"].astype(np.float32), g["p"], None)
    assert st.retcode == 0
    assert np.abs(logpx - g["logpx"]).max() < 1e-4 * np.abs(g["logpx"]).max()
    assert np.abs(zT - g["zT"]).max() < 1e-4 * np.abs(g["zT"]).max()
    dx, dp, sta = fj.backward_np(np.full(B, -1.0 / B, np.float32))
    assert sta.retcode_adj == 0
    assert _rel(dp, g["gp"]) < 5e-4 and _rel(dx, g["gx"]) < 5e-4


def test_multishoot_fixture_fp32():
    """multishoot.npz: the fused device loss (SSE, continuity term 100) 1e-5
    relative, the group predictions 1e-4, dL/dp through the discrete adjoint
    against the fixture's central differences 1e-3."""
    import torch

    import gbnde
    g = dict(np.load(os.path.join(GOLDEN, "multishoot.npz")))
    S, H = int(g["dims"][0]), int(g["dims"][1])
    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, S))
    pt = torch.tensor(g["p"], requires_grad=True)
    loss, preds = gbnde.multiple_shoot(pt, g["data"].astype(np.float32), g["ts"], model, gbnde.sse_loss,
                                       int(g["group_size"]), continuity_term=float(g["continuity_term"]),
                                       abstol=float(g["abstol"]), reltol=float(g["reltol"]))
    L = float(loss.detach())
    loss.backward()
    assert abs(L - float(g["loss"])) / float(g["loss"]) < 1e-5
    assert _rel(np.concatenate([np.asarray(a) for a in preds], axis=1), g["preds"]) < 1e-4
    assert _rel(pt.grad.numpy(), g["gp"]) < 1e-3
