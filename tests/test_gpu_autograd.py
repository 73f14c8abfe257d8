"""The torch autograd bridge keeps each call's own solve: a NeuralODE called
twice before backward (two batches in one loss, or one layer used twice in a
model) gets the gradient of both calls, not two copies of the last one.

The library's backward differentiates the context's last forward solve; the
bridge records which solve that was and solves a node's forward again when
another call has run since. Checked against the gradients of the two calls
taken one at a time (the solves are deterministic, so they agree to the last
bit up to the order of the final additions: 1e-6 relative)."""
import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("device", ["cuda", "cpu"])
def test_two_calls_before_backward(device):
    import torch

    import gbnde

    S, H, B = 4, 24, 40
    rng = np.random.default_rng(3)
    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, S))
    p0 = model.init_params(rng)
    ts = np.linspace(0.0, 1.0, 6)
    node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5(), saveat=ts, abstol=1e-6, reltol=1e-4)
    dev = torch.device(device, 0) if device == "cuda" else torch.device("cpu")
    xa = torch.from_numpy(rng.standard_normal((S, B)).astype(np.float32)).to(dev)
    xb = torch.from_numpy((2.0 * rng.standard_normal((S, B))).astype(np.float32)).to(dev)
    wa = torch.from_numpy(rng.standard_normal((S, B, len(ts))).astype(np.float32)).to(dev)
    wb = torch.from_numpy(rng.standard_normal((S, B, len(ts))).astype(np.float32)).to(dev)

    def one(x, w):
        p = torch.from_numpy(p0.copy()).to(dev).requires_grad_(True)
        xx = x.clone().requires_grad_(True)
        sol, _ = node(xx, p, None)
        (sol.array() * w).sum().backward()
        return p.grad.cpu().numpy(), xx.grad.cpu().numpy()

    gpa, gxa = one(xa, wa)
    gpb, gxb = one(xb, wb)

    p = torch.from_numpy(p0.copy()).to(dev).requires_grad_(True)
    xa2 = xa.clone().requires_grad_(True)
    xb2 = xb.clone().requires_grad_(True)
    sa, _ = node(xa2, p, None)
    sb, _ = node(xb2, p, None)   # a second solve on the same context before backward
    ((sa.array() * wa).sum() + (sb.array() * wb).sum()).backward()
    assert _rel(p.grad.cpu().numpy(), gpa + gpb) < 1e-6
    assert _rel(xa2.grad.cpu().numpy(), gxa) < 1e-6
    assert _rel(xb2.grad.cpu().numpy(), gxb) < 1e-6


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_stats_name_the_kernels_that_ran(precision):
    """gbnde_stats.fwd_path / adj_path: a BF16 context reports the tensor-core
    kernels for the NeuralODE solve and its InterpolatingAdjoint, and the FP32
    kernels for BacksolveAdjoint (which has no tensor-core form)."""
    import gbnde
    from gbnde import _lib

    S, H, B = 64, 256, 256
    rng = np.random.default_rng(5)
    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, H, "tanh"), gbnde.Dense(H, S))
    p = model.init_params(rng)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, 4)
    tc = precision == "bf16"
    for sense, want in ((gbnde.InterpolatingAdjoint(), _lib.PATH_TC if tc else _lib.PATH_FP32),
                        (gbnde.BacksolveAdjoint(), _lib.PATH_FP32)):
        node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5(precision), saveat=ts, abstol=1e-6,
                               reltol=1e-4, sensealg=sense)
        s = node.solver
        s.set_params(p)
        us, st = s.forward(u0, node.desc())
        assert st.fwd_path == (_lib.PATH_TC if tc else _lib.PATH_FP32)
        _, _, sta = s.backward(np.ones_like(us))
        assert sta.adj_path == want, (precision, sense, sta.adj_path)
        s.close()
