"""Packed multiple shooting (per-segment controllers in one launch) against the
FP64 oracle restatement of src/multiple_shooting.jl, through the C ABI.

Tolerances (relative): group predictions 1e-4 (FP32 kernel vs FP64 oracle,
both adaptive at 1e-8); loss 1e-5; gradient (discrete adjoint of the kernel vs
central differences of the oracle loss) 1e-3."""
import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def _problem(S, H, n, seed):
    import gbnde
    from oracle import tsit5 as ots
    rng = np.random.default_rng(seed)
    W = rng.standard_normal((S, S)) / np.sqrt(S)

    class Osc:  # damped oscillator network du/dt = -0.1 u + W tanh(u)
        def f(self, u, t):
            return -0.1 * u + W @ np.tanh(u)

    ts = 0.05 * np.arange(n)
    data, _ = ots.solve_forward(Osc(), rng.standard_normal((S, 1)), ts[0], ts[-1], ts, 1e-10, 1e-10)
    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, S))
    p = model.init_params(rng)
    return model, p, data[:, 0, :].astype(np.float32), ts


def _oracle_loss(model, p, trajectories, tol):
    from oracle import mlp as omlp
    from oracle import multishoot as oms
    om = omlp.MLP(model.dims, model.acts)
    total = 0.0
    allpreds = []
    for data, ts, gs in trajectories:
        rhs = omlp.MLPRHS(om, np.asarray(p, np.float64))
        preds, ok = oms.solve_groups(rhs, data.astype(np.float64), ts, gs, tol, tol)
        assert ok
        total += oms.multiple_shoot_loss(preds, data.astype(np.float64), gs, 100.0)
        allpreds += preds
    return total, allpreds


def test_single_trajectory_predictions_loss_gradient():
    import torch

    import gbnde
    S, H = 3, 8
    model, p, data, ts = _problem(S, H, 25, 0)
    tol = 1e-8
    sse = lambda u, uh: ((u - uh) ** 2).sum()  # noqa: E731
    pt = torch.tensor(p, requires_grad=True)
    loss, preds = gbnde.multiple_shoot(pt, data, ts, model, sse, 5, abstol=tol, reltol=tol)
    L0, opreds = _oracle_loss(model, p, [(data, ts, 5)], tol)
    assert len(preds) == len(opreds) == len(gbnde.group_ranges(25, 5))
    for a, b in zip(preds, opreds):
        assert _rel(a.detach().numpy(), b) < 1e-4
    assert abs(float(loss.detach()) - L0) / L0 < 1e-5
    loss.backward()
    eps = 1e-5
    fd = np.zeros(p.size)
    for i in range(p.size):
        e = np.zeros(p.size)
        e[i] = eps
        fd[i] = (_oracle_loss(model, p + e, [(data, ts, 5)], tol)[0] -
                 _oracle_loss(model, p - e, [(data, ts, 5)], tol)[0]) / (2 * eps)
    assert _rel(pt.grad.numpy(), fd) < 1e-3


def test_batched_uneven_segments_in_one_launch():
    import gbnde
    S, H = 4, 16
    rng = np.random.default_rng(5)
    model, p, _, _ = _problem(S, H, 10, 1)
    trajs = []
    for k in range(8):
        n = int(rng.integers(10, 41))
        gs = int(rng.integers(3, 9))
        _, _, data, ts = _problem(S, H, n, 100 + k)
        trajs.append((data, ts, gs))
    tol = 1e-8
    mse = lambda u, uh: float(np.mean((u - uh) ** 2))  # noqa: E731
    loss, preds = gbnde.multiple_shoot_batch(p, trajs, model, mse, abstol=tol, reltol=tol)
    from oracle import mlp as omlp
    from oracle import multishoot as oms
    om = omlp.MLP(model.dims, model.acts)
    k = 0
    Lref = 0.0
    for data, ts, gs in trajs:
        opreds, ok = oms.solve_groups(omlp.MLPRHS(om, p.astype(np.float64)), data.astype(np.float64), ts, gs,
                                      tol, tol)
        for b in opreds:
            assert _rel(preds[k], b) < 1e-4
            k += 1
        Lref += oms.multiple_shoot_loss(opreds, data.astype(np.float64), gs, 100.0,
                                        lambda u, uh: float(np.mean((u - uh) ** 2)))
    assert k == len(preds)
    assert abs(loss - Lref) / Lref < 1e-4


def test_failed_group_gives_inf_loss():
    import gbnde
    model, p, data, ts = _problem(3, 8, 20, 2)
    sse = lambda u, uh: float(np.sum((u - uh) ** 2))  # noqa: E731
    loss, preds = gbnde.multiple_shoot(p, data, ts, model, sse, 5, abstol=1e-12, reltol=1e-12, maxiters=2)
    assert loss == float("inf")


def test_config4_structure_uneven_batch():
    """cfg4 structure: state 32, MLP 32 -> 128 -> 128 -> 32 tanh (24,864
    parameters), data from du/dt = -0.1 u + W tanh(u), trajectories of uneven
    length (points at dt = 0.05) with their own group sizes, all segments in
    one launch; predictions and loss against the FP64 oracle."""
    import gbnde
    from oracle import mlp as omlp
    from oracle import multishoot as oms
    from oracle import tsit5 as ots
    S, H = 32, 128
    rng = np.random.default_rng(21)
    W = rng.standard_normal((S, S)) / np.sqrt(S)

    class Osc:
        def f(self, u, t):
            return -0.1 * u + W @ np.tanh(u)

    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, H, "tanh"), gbnde.Dense(H, S))
    p = model.init_params(rng)
    assert p.size == 24864
    trajs = []
    for k in range(6):
        n = int(rng.integers(40, 121))
        gs = int(rng.integers(5, 41))
        ts = 0.05 * np.arange(n)
        data, _ = ots.solve_forward(Osc(), rng.standard_normal((S, 1)), ts[0], ts[-1], ts, 1e-10, 1e-10)
        trajs.append((data[:, 0, :].astype(np.float32), ts, gs))
    tol = 1e-7
    mse = lambda u, uh: float(np.mean((u - uh) ** 2))  # noqa: E731
    loss, preds = gbnde.multiple_shoot_batch(p, trajs, model, mse, abstol=tol, reltol=tol)
    om = omlp.MLP(model.dims, model.acts)
    k = 0
    Lref = 0.0
    for data, ts, gs in trajs:
        opreds, ok = oms.solve_groups(omlp.MLPRHS(om, p.astype(np.float64)), data.astype(np.float64), ts, gs,
                                      tol, tol)
        assert ok
        for b in opreds:
            assert _rel(preds[k], b) < 1e-4
            k += 1
        Lref += oms.multiple_shoot_loss(opreds, data.astype(np.float64), gs, 100.0, mse)
    assert k == len(preds)
    assert abs(loss - Lref) / Lref < 1e-4


def _uneven_trajs(S, H, ntraj, seed):
    rng = np.random.default_rng(seed)
    model, p, _, _ = _problem(S, H, 10, seed)
    trajs = []
    for k in range(ntraj):
        n = int(rng.integers(10, 41))
        gs = int(rng.integers(3, 9))
        _, _, data, ts = _problem(S, H, n, 1000 * seed + k)
        trajs.append((data, ts, gs))
    return model, p, trajs


@pytest.mark.parametrize("kind", ["mse", "sse"])
@pytest.mark.parametrize("device", ["cpu", "cuda"])
def test_fused_device_loss_matches_host_loop_and_oracle(kind, device):
    """loss_function = mse_loss / sse_loss with the default continuity loss: the
    loss and its cotangent in one device kernel (gbnde_multishoot_loss), the
    adjoint from that cotangent. Against the host loop over groups (torch, same
    kernels): loss 1e-6, gradient 1e-5 relative; against the FP64 oracle's loss
    (src/multiple_shooting.jl:69-81): 1e-4."""
    import torch

    import gbnde
    from oracle import mlp as omlp
    from oracle import multishoot as oms
    S, H = 4, 16
    model, p, trajs = _uneven_trajs(S, H, 8, 3)
    solver = gbnde.Solver(model, "fp32", 0)
    tol = 1e-8
    lf = gbnde.mse_loss if kind == "mse" else gbnde.sse_loss
    host = (lambda u, uh: ((u - uh) ** 2).mean()) if kind == "mse" else (lambda u, uh: ((u - uh) ** 2).sum())
    dev = torch.device(device, 0) if device == "cuda" else torch.device("cpu")
    pf = torch.tensor(p, device=dev, requires_grad=True)
    # the fused path keeps the saves on the device: `early` is read right
    # after the call (gbnde_multishoot_saves), `preds` only after another solve
    # ran on the context (the forward is solved again)
    _, early = gbnde.multiple_shoot_batch(pf, trajs, solver, lf, abstol=tol, reltol=tol)
    early = [np.asarray(a).copy() for a in early]
    Lf, preds = gbnde.multiple_shoot_batch(pf, trajs, solver, lf, abstol=tol, reltol=tol)
    Lf.backward()
    ph = torch.tensor(p, requires_grad=True)
    Lh, preds_h = gbnde.multiple_shoot_batch(ph, trajs, solver, host, abstol=tol, reltol=tol)
    Lh.backward()
    Lf, Lh = float(Lf.detach()), float(Lh.detach())
    assert abs(Lf - Lh) / abs(Lh) < 1e-6
    assert _rel(pf.grad.cpu().numpy(), ph.grad.numpy()) < 1e-5
    assert len(preds) == len(preds_h) == len(early)
    for a, b, c in zip(preds, preds_h, early):
        assert np.array_equal(np.asarray(a), b.detach().numpy())
        assert np.array_equal(c, b.detach().numpy())
    om = omlp.MLP(model.dims, model.acts)
    ofn = (lambda u, uh: float(np.mean((u - uh) ** 2))) if kind == "mse" else None
    Lref = 0.0
    for data, ts, gs in trajs:
        opreds, ok = oms.solve_groups(omlp.MLPRHS(om, p.astype(np.float64)), data.astype(np.float64), ts, gs,
                                      tol, tol)
        assert ok
        Lref += oms.multiple_shoot_loss(opreds, data.astype(np.float64), gs, 100.0, ofn)
    assert abs(float(Lf) - Lref) / Lref < 1e-4
    solver.close()


def test_fused_loss_gradient_against_finite_differences_and_failure():
    """The fused path's gradient against central differences of the oracle's
    multiple-shooting loss (1e-3), and a failed group still gives Inf."""
    import torch

    import gbnde
    S, H = 3, 8
    model, p, data, ts = _problem(S, H, 25, 0)
    tol = 1e-8
    pt = torch.tensor(p, requires_grad=True)
    loss, preds = gbnde.multiple_shoot(pt, data, ts, model, gbnde.sse_loss, 5, abstol=tol, reltol=tol)
    L0, _ = _oracle_loss(model, p, [(data, ts, 5)], tol)
    assert abs(float(loss.detach()) - L0) / L0 < 1e-5
    loss.backward()
    eps = 1e-5
    fd = np.zeros(p.size)
    for i in range(p.size):
        e = np.zeros(p.size)
        e[i] = eps
        fd[i] = (_oracle_loss(model, p + e, [(data, ts, 5)], tol)[0] -
                 _oracle_loss(model, p - e, [(data, ts, 5)], tol)[0]) / (2 * eps)
    assert _rel(pt.grad.numpy(), fd) < 1e-3
    loss, preds = gbnde.multiple_shoot(p, data, ts, model, gbnde.sse_loss, 5, abstol=1e-12, reltol=1e-12,
                                       maxiters=2)
    assert loss == float("inf")
