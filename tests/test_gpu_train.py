"""One training iteration through gbnde_train_step (forward, fused loss,
adjoint gradient, Adam on the device parameters) against the same pieces
called one by one with a numpy Adam, and a short training run whose loss
goes down. Both precision forms."""
import numpy as np
import pytest

from conftest import gpu_available
from test_gpu_neural_ode import _setup

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]


def _problem(prec, S=16, H=64, B=256, nsave=8, seed=11):
    import torch

    import gbnde
    model, p, rng = _setup([S, H, H, S], ["tanh", "tanh", "identity"], False, B, seed, bias=0.01)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, nsave)
    M = -0.5 * np.eye(S) + 0.1 * rng.standard_normal((S, S))
    from scipy.linalg import expm
    tgt = np.stack([expm(M * t) @ u0.astype(np.float64) for t in ts], axis=-1).astype(np.float32)
    solver = gbnde.Solver(model, prec, 0)
    desc = gbnde.Solver.solve_desc(0.0, 1.0, ts, 1e-6, 1e-4, 0)
    dev = torch.device("cuda", 0)
    u0_d = torch.from_numpy(np.ascontiguousarray(u0.T)).to(dev)                     # column-major S x B
    tg_d = torch.from_numpy(np.ascontiguousarray(np.transpose(tgt, (2, 1, 0)))).to(dev)
    return solver, desc, u0_d, tg_d, torch.from_numpy(p.copy()).to(dev), S, B, nsave


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_train_step_matches_pieces_and_numpy_adam(prec):
    import torch
    solver, desc, u0_d, tg_d, p_d, S, B, ns = _problem(prec)
    dev = p_d.device
    lr, b1, b2, eps = 1e-3, 0.9, 0.999, 1e-8
    # reference: the library's own gradient, then Adam in FP64 numpy
    solver.set_params_device(p_d)
    us = torch.empty((ns, B, S), dtype=torch.float32, device=dev)
    dl = torch.empty_like(us)
    du0 = torch.empty((B, S), dtype=torch.float32, device=dev)
    dp = torch.empty_like(p_d)
    st = solver.forward_device(u0_d, us, desc, S, B)
    assert st.retcode == 0
    loss_ref = solver.loss_device(us, tg_d, 1, dl)
    sb = solver.backward_device(dl, du0, dp)
    assert sb.retcode_adj == 0
    g = dp.double().cpu().numpy()
    p0 = p_d.double().cpu().numpy()
    m = np.zeros_like(g)
    v = np.zeros_like(g)
    p_ref = p0.copy()
    for step in (1, 2):
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        mh = m / (1 - b1 ** step)
        vh = v / (1 - b2 ** step)
        p_ref = p_ref - lr * mh / (np.sqrt(vh) + eps)
        if step == 1:
            p_ref1 = p_ref.copy()
    # the fused step, twice on the same data (the second uses the new params)
    pt = p_d.clone()
    mt = torch.zeros_like(pt)
    vt = torch.zeros_like(pt)
    loss1, st1 = solver.train_step(u0_d, tg_d, desc, S, B, pt, mt, vt, 1, lr, b1, b2, eps, kind=1)
    assert st1.retcode == 0 and st1.retcode_adj == 0
    assert abs(loss1 - loss_ref) <= 1e-12 * max(1.0, abs(loss_ref))
    assert np.abs(pt.double().cpu().numpy() - p_ref1).max() <= 1e-3 * lr
    np.testing.assert_allclose(mt.double().cpu().numpy(), (1 - b1) * g, rtol=1e-6, atol=1e-12)
    loss2, st2 = solver.train_step(u0_d, tg_d, desc, S, B, pt, mt, vt, 2, lr, b1, b2, eps, kind=1)
    assert st2.retcode == 0 and np.isfinite(loss2)
    # the context now holds the updated parameters
    us2 = torch.empty_like(us)
    solver.forward_device(u0_d, us2, desc, S, B)
    dl2 = torch.empty_like(us)
    loss_after = solver.loss_device(us2, tg_d, 1, dl2)
    assert loss_after < loss1


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_training_reduces_the_loss(prec):
    import torch
    solver, desc, u0_d, tg_d, p_d, S, B, ns = _problem(prec, seed=3)
    m = torch.zeros_like(p_d)
    v = torch.zeros_like(p_d)
    losses = []
    for step in range(1, 31):
        loss, st = solver.train_step(u0_d, tg_d, desc, S, B, p_d, m, v, step, lr=3e-3, kind=1)
        assert st.retcode == 0 and st.retcode_adj == 0
        losses.append(loss)
    assert losses[-1] < 0.7 * losses[0], losses[::5]


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_graph_train_step_replays_the_eager_step(prec):
    """gbnde_graph_train_step: the first call runs eagerly and captures the
    iteration; later calls replay the graph. The parameter trajectory and the
    losses equal those of eager gbnde_train_step on the same data."""
    import torch
    solver, desc, u0_d, tg_d, p0, S, B, ns = _problem(prec, seed=5)
    solver_e, desc_e, _, _, _, _, _, _ = _problem(prec, seed=5)
    pg, mg, vg = p0.clone(), torch.zeros_like(p0), torch.zeros_like(p0)
    pe, me, ve = p0.clone(), torch.zeros_like(p0), torch.zeros_like(p0)
    graphed = []
    for step in range(1, 7):
        lg, sg, g = solver.graph_train_step(u0_d, tg_d, desc, S, B, pg, mg, vg, step, lr=2e-3, kind=1)
        le, se = solver_e.train_step(u0_d, tg_d, desc_e, S, B, pe, me, ve, step, lr=2e-3, kind=1)
        assert sg.retcode == 0 and sg.retcode_adj == 0
        assert abs(lg - le) <= 1e-9 * abs(le), (step, lg, le)
        assert sg.nf == se.nf and sg.nf_adj == se.nf_adj
        assert torch.equal(pg, pe), step
        graphed.append(g)
    assert graphed[0] is False
    assert all(graphed[1:]), graphed


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_autotune_keeps_results(prec):
    """gbnde_autotune times the kernels at each tile size and keeps the
    fastest; solves after it give the same states and gradients as before
    (within FP32 reduction-order noise)."""
    import torch
    solver, desc, u0_d, tg_d, p_d, S, B, ns = _problem(prec, B=1000, seed=3)
    dev = p_d.device
    solver.set_params_device(p_d)

    def run():
        us = torch.empty((ns, B, S), dtype=torch.float32, device=dev)
        dl = torch.empty_like(us)
        du0 = torch.empty((B, S), dtype=torch.float32, device=dev)
        dp = torch.empty_like(p_d)
        st = solver.forward_device(u0_d, us, desc, S, B)
        assert st.retcode == 0
        loss = solver.loss_device(us, tg_d, 1, dl)
        sb = solver.backward_device(dl, du0, dp)
        assert sb.retcode_adj == 0
        return us.double(), loss, du0.double(), dp.double()

    before = run()
    tiles = solver.autotune(u0_d, desc, S, B)
    if prec == "fp32":
        assert tiles[0] in (8, 16, 32, 64) and tiles[1] in (8, 16, 32, 64), tiles
    else:
        assert tiles[0] == 128 and tiles[1] in (0, 1), tiles
    after = run()
    assert abs(after[1] - before[1]) <= 1e-5 * abs(before[1])
    for a, b in zip((after[0], after[2], after[3]), (before[0], before[2], before[3])):
        err = (a - b).norm().item() / b.norm().item()
        assert err <= 1e-4, err


def test_autotune_bf16_chooses_an_engine():
    """The BF16 form's autotuner times the single-accumulator and the stash
    tensor-core engines on a shape both cover and keeps the faster; the two
    engines give the same gradient to 1e-4 (the stash engine evaluates every
    adjoint stage in full, the other reuses stage 6's activations for stage 7)."""
    import torch

    import gbnde
    from gbnde import _lib
    S, H, B = 64, 256, 2048
    rng = np.random.default_rng(12)
    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, H, "tanh"), gbnde.Dense(H, S))
    p = model.init_params(rng)
    solver = gbnde.Solver(model, "bf16", 0)
    desc = gbnde.Solver.solve_desc(0.0, 1.0, np.linspace(0, 1, 6), 1e-7, 1e-5, 0)
    dev = torch.device("cuda", 0)
    u0 = torch.from_numpy(np.ascontiguousarray(rng.standard_normal((B, S)).astype(np.float32))).to(dev)
    us = torch.empty((6, B, S), dtype=torch.float32, device=dev)
    g = torch.from_numpy(rng.standard_normal((6, B, S)).astype(np.float32)).to(dev)
    du0 = torch.empty((B, S), dtype=torch.float32, device=dev)
    dp = torch.empty(solver.nparams, dtype=torch.float32, device=dev)
    solver.set_params(p)

    def grad():
        st = solver.forward_device(u0, us, desc, S, B)
        sb = solver.backward_device(g, du0, dp)
        torch.cuda.synchronize()
        assert st.fwd_path == _lib.PATH_TC and sb.adj_path == _lib.PATH_TC
        return dp.double().cpu().numpy(), du0.double().cpu().numpy()

    g0, u0g = grad()
    rows, engine = solver.autotune(u0, desc, S, B)
    assert rows == 128 and engine in (0, 1)
    g1, u1g = grad()
    assert np.linalg.norm(g1 - g0) <= 1e-4 * np.linalg.norm(g0)
    assert np.linalg.norm(u1g - u0g) <= 1e-4 * np.linalg.norm(u0g)
