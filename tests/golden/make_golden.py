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
"""
import os
import sys

import numpy as np
from scipy.linalg import expm

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import mlp as omlp  # noqa: E402
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


if __name__ == "__main__":
    spiral()
    linear()
    batched()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")
