"""CPU checks of the FFJORD oracle: the Hutchinson estimate averages to the
exact trace, and the adjoint gradient of logpx matches finite differences."""
import numpy as np

from oracle import ffjord as off
from oracle import mlp as omlp
from oracle import tsit5 as ots


def _solve(rhs, x, tol):
    d, B = x.shape
    y0 = np.vstack([x, np.zeros((1, B))])
    ys, integ = ots.solve_forward(rhs, y0, 0.0, 1.0, [1.0], tol, tol)
    return ys[..., 0], integ


def test_hutchinson_averages_to_exact_trace():
    rng = np.random.default_rng(0)
    m = omlp.MLP([3, 9, 2], ["softplus", "identity"], time_input=True)
    p = m.glorot_uniform(rng).astype(np.float64)
    z = rng.standard_normal((2, 5))
    y = np.vstack([z, np.zeros((1, 5))])
    exact = off.FFJORDRHS(m, p, exact=True).f(y, 0.2)[2]
    est = np.zeros(5)
    n = 4000
    for _ in range(n):
        e = rng.choice([-1.0, 1.0], size=(2, 5))
        est += off.FFJORDRHS(m, p, noise=e).f(y, 0.2)[2]
    assert np.abs(est / n - exact).max() < 0.05 * np.abs(exact).max() + 1e-3


def test_ffjord_adjoint_matches_finite_differences():
    rng = np.random.default_rng(1)
    d, B = 2, 3
    m = omlp.MLP([d + 1, 6, d], ["tanh", "identity"], time_input=True)
    p = m.glorot_uniform(rng).astype(np.float64)
    x = rng.standard_normal((d, B))
    e = rng.choice([-1.0, 1.0], size=(d, B))
    tol = 1e-10

    def nll(pp, xx):
        yT, _ = _solve(off.FFJORDRHS(m, pp, noise=e), xx, tol)
        return -np.mean(off.logpx_from_final(yT, d))

    rhs = off.FFJORDRHS(m, p, noise=e)
    yT, fwd = _solve(rhs, x, tol)
    g = -np.ones(B) / B                       # dL/dlogpx
    dy = np.vstack([-yT[:d] * g, -g[None, :]])
    gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, [1.0], dy[..., None], 0.0, tol, tol)
    eps = 1e-6
    fdp = np.array([(nll(p + eps * v, x) - nll(p - eps * v, x)) / (2 * eps) for v in np.eye(p.size)])
    fdx = np.zeros_like(x)
    for i in np.ndindex(x.shape):
        v = np.zeros_like(x)
        v[i] = eps
        fdx[i] = (nll(p, x + v) - nll(p, x - v)) / (2 * eps)
    assert np.linalg.norm(gp - fdp) / np.linalg.norm(fdp) < 1e-6
    assert np.linalg.norm(gu[:d] - fdx) / np.linalg.norm(fdx) < 1e-6
