"""Multi-rank paths on CPU with the gloo backend, world size 2, on real
problems (the FP64 oracle restatement computes every rank's share):

* multiple shooting sharded by trajectory (the groups of a trajectory stay on
  one rank, since the continuity term couples consecutive groups;
  src/multiple_shooting.jl:52-81): each rank sums the loss and gradient of its
  trajectories, one all-reduce sums them, and the result equals the
  single-process loss and gradient of all trajectories;
* replica data-parallel training: each rank solves its own batch (its own
  controller: the reference couples a batch through one step size,
  src/neural_de.jl:52), the gradients are averaged, and the Adam step leaves
  identical parameters on both ranks, equal to the single-process step over
  the same two replicas.
"""
import os
import socket

import numpy as np


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _setup_paths():
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for q in (root, os.path.join(root, "diffeqflux.jl_gb300")):
        if q not in sys.path:
            sys.path.insert(0, q)


# ---- problems (deterministic, built identically in every process) -------------
S, H = 3, 8
TOL = 1e-8


def _model_and_params(seed=0):
    from oracle import mlp as omlp
    om = omlp.MLP([S, H, S], ["tanh", "identity"])
    p = om.glorot_uniform(np.random.default_rng(seed)).astype(np.float64)
    return om, p


def _trajectories():
    from oracle import tsit5 as ots
    rng = np.random.default_rng(11)
    W = rng.standard_normal((S, S)) / np.sqrt(S)

    class Osc:  # du/dt = -0.1 u + W tanh(u)
        def f(self, u, t):
            return -0.1 * u + W @ np.tanh(u)

    out = []
    for k in range(5):
        n = int(rng.integers(8, 17))
        gs = int(rng.integers(3, 6))
        ts = 0.05 * np.arange(n)
        d, _ = ots.solve_forward(Osc(), rng.standard_normal((S, 1)), 0.0, ts[-1], ts, 1e-10, 1e-10)
        out.append((d[:, 0, :], ts, gs))
    return out


def _ms_loss_grad(om, p, trajs, cont=100.0):
    """Sum over trajectories of the multiple-shooting loss (per-group MSE plus
    the default continuity loss) and its gradient: every group's prediction
    cotangent through the oracle's InterpolatingAdjoint."""
    from oracle import mlp as omlp
    from oracle import multishoot as oms
    from oracle import tsit5 as ots
    rhs = omlp.MLPRHS(om, p)
    L, g = 0.0, np.zeros(p.size)
    for data, ts, gs in trajs:
        rngs = oms.group_ranges(data.shape[1], gs)
        sols = []
        for (a, b) in rngs:
            tsg = ts[a:b + 1]
            us, fwd = ots.solve_forward(rhs, data[:, a:a + 1], tsg[0], tsg[-1], tsg, TOL, TOL)
            sols.append((us[:, 0, :], fwd, tsg))
        cots = []
        for i, (a, b) in enumerate(rngs):
            pred = sols[i][0]
            u = data[:, a:b + 1]
            L += float(np.mean((u - pred) ** 2))
            cots.append(2.0 * (pred - u) / u.size)
            if i > 0:
                prev = sols[i - 1][0][:, -1]
                L += cont * float(np.sum(np.abs(prev - u[:, 0])))
                cots[i - 1][:, -1] += cont * np.sign(prev - u[:, 0])
        for (pred, fwd, tsg), cot in zip(sols, cots):
            _, gp, _ = ots.adjoint_interpolating(rhs, fwd, tsg, cot[:, None, :], tsg[0], TOL, TOL)
            g += gp
    return L, g


def _replica_grad(om, p, rank, B=6):
    from gbnde import replicas
    from oracle import mlp as omlp
    from oracle import tsit5 as ots
    rng = np.random.default_rng(replicas.replica_seed(3, rank))
    u0 = rng.standard_normal((S, B))
    ts = np.linspace(0.0, 1.0, 5)
    tg = 0.5 * rng.standard_normal((S, B, len(ts)))
    rhs = omlp.MLPRHS(om, p)
    us, fwd = ots.solve_forward(rhs, u0, 0.0, 1.0, ts, 1e-7, 1e-5)
    _, gp, _ = ots.adjoint_interpolating(rhs, fwd, ts, 2.0 * (us - tg) / us.size, 0.0, 1e-7, 1e-5)
    return gp


def _adam(p, g, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    return p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps), m, v


def _worker(rank, world, port, q):
    _setup_paths()
    import torch.distributed as dist

    from gbnde import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    om, p = _model_and_params()
    trajs = _trajectories()
    mine = [trajs[i] for i in replicas.shard_segments(len(trajs), rank, world)]
    L, g = _ms_loss_grad(om, p, mine)
    Ls = replicas.sum_over_ranks(L)
    gs = replicas.sum_over_ranks(g)
    # two data-parallel Adam steps on replica batches
    pr, m, v = p.copy(), np.zeros_like(p), np.zeros_like(p)
    for step in (1, 2):
        gr = replicas.average_gradients(_replica_grad(om, pr, rank))
        pr, m, v = _adam(pr, gr, m, v, step)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, len(mine), Ls, gs, pr))


def test_sharded_multiple_shooting_and_replica_training_gloo_world2():
    import multiprocessing as mp
    _setup_paths()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted([q.get(timeout=300) for _ in ps], key=lambda x: x[0])
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    # single process: all trajectories, and both replicas
    om, p = _model_and_params()
    L1, g1 = _ms_loss_grad(om, p, _trajectories())
    assert out[0][1] + out[1][1] == 5 and min(out[0][1], out[1][1]) >= 2
    for r in range(2):
        assert abs(out[r][2] - L1) <= 1e-12 * abs(L1)
        assert np.linalg.norm(out[r][3] - g1) <= 1e-10 * np.linalg.norm(g1)
    pr, m, v = p.copy(), np.zeros_like(p), np.zeros_like(p)
    for step in (1, 2):
        gr = 0.5 * (_replica_grad(om, pr, 0) + _replica_grad(om, pr, 1))
        pr, m, v = _adam(pr, gr, m, v, step)
    assert np.array_equal(out[0][4], out[1][4])          # replicas stay in lockstep
    assert np.linalg.norm(out[0][4] - pr) <= 1e-12 * np.linalg.norm(pr)
    assert np.linalg.norm(pr - p) > 0


def test_sharded_gradient_matches_finite_differences():
    """The oracle multiple-shooting gradient used above, against central differences."""
    _setup_paths()
    om, p = _model_and_params()
    trajs = _trajectories()[:2]
    L, g = _ms_loss_grad(om, p, trajs)
    rng = np.random.default_rng(0)
    for i in rng.choice(p.size, 6, replace=False):
        e = np.zeros(p.size)
        e[i] = 1e-6
        fd = (_ms_loss_grad(om, p + e, trajs)[0] - _ms_loss_grad(om, p - e, trajs)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(g).max())
