"""Generates the golden fixtures under tests/golden/ with the FP64 oracle.

Run from the repository root:  python tests/golden/make_golden.py

Each fixture holds seeded inputs (initial states, flat Lux-order parameters,
save times, tolerances, loss cotangents) and the oracle's outputs (saved
states, dL/du0 and dL/dp for InterpolatingAdjoint and BacksolveAdjoint), so
that any implementation -- this library's kernels, or a Julia session running
the reference -- can be checked on identical inputs.

  spiral.npz   the spiral NeuralODE (docs/src/examples/neural_ode.md:19-36):
               u0=[2,0], tspan (0,1.5), 30 save points, cube -> Dense(2,50,tanh)
               -> Dense(50,2), abstol 1e-7 reltol 1e-5, SSE loss against the
               cubic spiral data solved at 1e-10.
  linear.npz   known answer: one identity Dense layer, du/dt = W u, exact
               solution expm(W t) u0 at 11 save points.
  batched.npz  state 16, MLP 16->64->64->16 tanh, 8 trajectories, 20 save
               points, abstol 1e-7 reltol 1e-5, MSE loss (the headline configuration's
               structure at a size that keeps the fixture small).
  ffjord.npz   FFJORD with the exact trace (monte_carlo = false, deterministic in
               the reference too; src/ffjord.jl:120-129), d = 2, model
               Dense(2,16,tanh) -> Dense(16,2) without a time input, 16 samples,
               tspan (0,1), 1e-8 / 1e-8: logpx, z(t1), and the gradients of
               -mean(logpx) with respect to p and x (the oracle's adjoint, checked
               here against central differences).
  multishoot.npz  multiple_shoot of one trajectory (src/multiple_shooting.jl:36-94):
               state 2, 21 data points at dt = 0.1 from du/dt = A u^3, model
               Dense(2,16,tanh) -> Dense(16,2), group size 5, continuity_term 100,
               SSE loss, 1e-8 / 1e-8: the loss, the group predictions, and dL/dp by
               central differences of the oracle's loss.
"""
import os
import sys

import numpy as np
from scipy.linalg import expm

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ffjord as off  # noqa: E402
from oracle import mlp as omlp  # noqa: E402
from oracle import multishoot as oms  # noqa: E402
from oracle import tsit5 as ots  # noqa: E402


def _grads(rhs, fwd, usave, ts, dL, t0, abstol, reltol):
    gu, gp, bi = ots.adjoint_interpolating(rhs, fwd, ts, dL, t0, abstol, reltol)
    gu2, gp2, bb = ots.adjoint_backsolve(rhs, usave, ts, dL, t0, abstol, reltol)
    return gu, gp, gu2, gp2


def spiral():
    rng = np.random.default_rng(0)
    m = omlp.MLP([2, 50, 2], ["tanh", "identity"], cube_input=True)
    p = m.glorot_uniform(rng).astype(np.float32)
    u0 = np.array([[2.0], [0.0]])
    ts = np.linspace(0.0, 1.5, 30)
    A = np.array([[-0.1, 2.0], [-2.0, -0.1]])

    class Spiral:
        def f(self, u, t):
            return ((u ** 3).T @ A).T

    data, _ = ots.solve_forward(Spiral(), u0, 0.0, 1.5, ts, 1e-10, 1e-10)
    rhs = omlp.MLPRHS(m, p.astype(np.float64))
    us, fwd = ots.solve_forward(rhs, u0, 0.0, 1.5, ts, 1e-7, 1e-5)
    dL = 2.0 * (us - data)
    gu, gp, gu2, gp2 = _grads(rhs, fwd, us, ts, dL, 0.0, 1e-7, 1e-5)
    np.savez(os.path.join(HERE, "spiral.npz"), dims=np.array([2, 50, 2]), cube=1, p=p, u0=u0,
             ts=ts, abstol=1e-7, reltol=1e-5, data=data, usave=us, loss=np.sum((us - data) ** 2),
             dLdu=dL, gu_interp=gu, gp_interp=gp, gu_back=gu2, gp_back=gp2,
             naccept=fwd.naccept, nreject=fwd.nreject)


def linear():
    rng = np.random.default_rng(1)
    S, B = 6, 4
    Q, _ = np.linalg.qr(rng.standard_normal((S, S)))
    W = Q @ np.diag(-rng.uniform(0.1, 2.0, S)) @ Q.T + 0.3 * (rng.standard_normal((S, S)) - 0.0) * 0.1
    m = omlp.MLP([S, S], ["identity"])
    p = m.flatten([(W, np.zeros(S))]).astype(np.float32)
    W32 = m.unflatten(p.astype(np.float64))[0][0]
    u0 = rng.standard_normal((S, B)).astype(np.float32).astype(np.float64)
    ts = np.linspace(0.0, 1.0, 11)
    exact = np.stack([expm(W32 * t) @ u0 for t in ts], axis=-1)
    rhs = omlp.MLPRHS(m, p.astype(np.float64))
    us, fwd = ots.solve_forward(rhs, u0, 0.0, 1.0, ts, 1e-9, 1e-9)
    np.savez(os.path.join(HERE, "linear.npz"), dims=np.array([S, S]), cube=0, p=p, u0=u0, ts=ts,
             abstol=1e-9, reltol=1e-9, exact=exact, usave=us)


def batched():
    rng = np.random.default_rng(2)
    S, H, B = 16, 64, 8
    m = omlp.MLP([S, H, H, S], ["tanh", "tanh", "identity"])
    p = m.glorot_uniform(rng).astype(np.float32)
    u0 = rng.standard_normal((S, B)).astype(np.float32).astype(np.float64)
    ts = np.linspace(0.0, 1.0, 20)
    rhs = omlp.MLPRHS(m, p.astype(np.float64))
    us, fwd = ots.solve_forward(rhs, u0, 0.0, 1.0, ts, 1e-7, 1e-5)
    tgt = 0.5 * rng.standard_normal(us.shape)
    dL = 2.0 * (us - tgt) / us.size
    gu, gp, gu2, gp2 = _grads(rhs, fwd, us, ts, dL, 0.0, 1e-7, 1e-5)
    np.savez(os.path.join(HERE, "batched.npz"), dims=np.array([S, H, H, S]), cube=0, p=p, u0=u0,
             ts=ts, abstol=1e-7, reltol=1e-5, target=tgt, usave=us, loss=np.mean((us - tgt) ** 2),
             dLdu=dL, gu_interp=gu, gp_interp=gp, gu_back=gu2, gp_back=gp2,
             naccept=fwd.naccept, nreject=fwd.nreject)


def ffjord():
    rng = np.random.default_rng(3)
    d, H, B, tol = 2, 16, 16, 1e-8
    m = omlp.MLP([d, H, d], ["tanh", "identity"])
    p = m.glorot_uniform(rng).astype(np.float32)
    x = (rng.standard_normal((d, B)) * 0.7 + rng.choice([-1.0, 1.0], size=(1, B))).astype(np.float32)
    x = x.astype(np.float64)

    def solve(pp, xx):
        rhs = off.FFJORDRHS(m, pp, exact=True)
        ys, fwd = ots.solve_forward(rhs, np.vstack([xx, np.zeros((1, B))]), 0.0, 1.0, [1.0], tol, tol)
        return rhs, ys[..., 0], fwd

    rhs, yT, fwd = solve(p.astype(np.float64), x)
    logpx = off.logpx_from_final(yT, d)
    g = -np.ones(B) / B                      # dL/dlogpx of L = -mean(logpx)
    dy = np.vstack([-yT[:d] * g, -g[None, :]])
    gx, gp, _ = ots.adjoint_interpolating(rhs, fwd, [1.0], dy[..., None], 0.0, tol, tol)
    nll = lambda pp, xx: -np.mean(off.logpx_from_final(solve(pp, xx)[1], d))  # noqa: E731
    eps = 1e-6
    p64 = p.astype(np.float64)
    fdp = np.array([(nll(p64 + eps * v, x) - nll(p64 - eps * v, x)) / (2 * eps) for v in np.eye(p.size)])
    assert np.linalg.norm(gp - fdp) / np.linalg.norm(fdp) < 1e-5
    np.savez(os.path.join(HERE, "ffjord.npz"), dims=np.array([d, H, d]), p=p, x=x, tspan=np.array([0.0, 1.0]),
             abstol=tol, reltol=tol, logpx=logpx, zT=yT[:d], delta_logp=yT[d], gp=gp, gx=gx[:d],
             naccept=fwd.naccept, nreject=fwd.nreject)


def multishoot():
    rng = np.random.default_rng(4)
    S, H, n, gs, tol = 2, 16, 21, 5, 1e-8
    A = np.array([[-0.1, 2.0], [-2.0, -0.1]])

    class Cubic:
        def f(self, u, t):
            return ((u ** 3).T @ A).T

    ts = 0.1 * np.arange(n)
    data, _ = ots.solve_forward(Cubic(), np.array([[2.0], [0.0]]), 0.0, ts[-1], ts, 1e-10, 1e-10)
    data = data[:, 0, :].astype(np.float32).astype(np.float64)
    m = omlp.MLP([S, H, S], ["tanh", "identity"])
    p = m.glorot_uniform(rng).astype(np.float32)

    def loss(pp):
        preds, ok = oms.solve_groups(omlp.MLPRHS(m, pp), data, ts, gs, tol, tol)
        assert ok
        return oms.multiple_shoot_loss(preds, data, gs, 100.0), preds

    p64 = p.astype(np.float64)
    L, preds = loss(p64)
    eps = 1e-6
    gp = np.array([(loss(p64 + eps * v)[0] - loss(p64 - eps * v)[0]) / (2 * eps) for v in np.eye(p.size)])
    np.savez(os.path.join(HERE, "multishoot.npz"), dims=np.array([S, H, S]), p=p, data=data, ts=ts,
             group_size=gs, continuity_term=100.0, abstol=tol, reltol=tol, loss=L,
             preds=np.concatenate(preds, axis=1), gp=gp)


if __name__ == "__main__":
    spiral()
    linear()
    batched()
    ffjord()
    multishoot()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")
