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


def _solve_reg(rhs, x, tol):
    d, B = x.shape
    y0 = np.vstack([x, np.zeros((3, B))])
    ys, integ = ots.solve_forward(rhs, y0, 0.0, 1.0, [1.0], tol, tol)
    return ys[..., 0], integ


def test_regularizer_rows_against_a_finite_difference_jacobian():
    """regularize = true (src/ffjord.jl:131-132): the extra rows are |f|^2 and
    |e^T J| with J = df/dz taken here by central differences."""
    rng = np.random.default_rng(2)
    d, B = 3, 4
    m = omlp.MLP([d + 1, 7, d], ["tanh", "identity"], time_input=True)
    p = m.glorot_uniform(rng).astype(np.float64)
    z = rng.standard_normal((d, B))
    e = rng.standard_normal((d, B))
    y = np.vstack([z, np.zeros((3, B))])
    for exact in (False, True):
        g = off.FFJORDRHS(m, p, noise=e, exact=exact, regularize=True).f(y, 0.3)
        f = m.forward(p, z, 0.3)
        assert np.allclose(g[:d], f) and np.allclose(g[d + 1], np.sum(f * f, axis=0))
        eps = 1e-6
        J = np.zeros((B, d, d))
        for k in range(d):
            dz = np.zeros_like(z)
            dz[k] = eps
            J[:, :, k] = ((m.forward(p, z + dz, 0.3) - m.forward(p, z - dz, 0.3)) / (2 * eps)).T
        eJ = np.einsum("bi,bik->bk", e.T, J)
        assert np.allclose(g[d + 2], np.linalg.norm(eJ, axis=1), rtol=1e-7, atol=1e-9)
        tr = np.trace(J, axis1=1, axis2=2) if exact else np.einsum("bi,bik,bk->b", e.T, J, e.T)
        assert np.allclose(-g[d], tr, rtol=1e-7, atol=1e-9)


def test_regularized_adjoint_matches_finite_differences():
    """Gradient of -mean(logpx) + a mean(lambda1) + b mean(lambda2) through the
    regularised system, Hutchinson and exact trace."""
    rng = np.random.default_rng(3)
    d, B = 2, 3
    m = omlp.MLP([d + 1, 6, d], ["tanh", "identity"], time_input=True)
    p = m.glorot_uniform(rng).astype(np.float64)
    x = rng.standard_normal((d, B))
    e = rng.choice([-1.0, 1.0], size=(d, B))
    tol = 1e-10
    wa, wb = 0.7, 1.3
    for exact in (False, True):
        def loss(pp, xx):
            yT, _ = _solve_reg(off.FFJORDRHS(m, pp, noise=e, exact=exact, regularize=True), xx, tol)
            return -np.mean(off.logpx_from_final(yT, d)) + wa * np.mean(yT[d + 1]) + wb * np.mean(yT[d + 2])

        rhs = off.FFJORDRHS(m, p, noise=e, exact=exact, regularize=True)
        yT, fwd = _solve_reg(rhs, x, tol)
        g = -np.ones(B) / B
        dy = np.vstack([-yT[:d] * g, -g[None, :], np.full((1, B), wa / B), np.full((1, B), wb / B)])
        gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, [1.0], dy[..., None], 0.0, tol, tol)
        eps = 1e-6
        fdp = np.array([(loss(p + eps * v, x) - loss(p - eps * v, x)) / (2 * eps) for v in np.eye(p.size)])
        fdx = np.zeros_like(x)
        for i in np.ndindex(x.shape):
            v = np.zeros_like(x)
            v[i] = eps
            fdx[i] = (loss(p, x + v) - loss(p, x - v)) / (2 * eps)
        assert np.linalg.norm(gp - fdp) / np.linalg.norm(fdp) < 1e-6
        assert np.linalg.norm(gu[:d] - fdx) / np.linalg.norm(fdx) < 1e-6
