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
