"""FFJORD (FP32 form) against the FP64 oracle through the C ABI: logpx with the
Hutchinson and the exact trace, and the InterpolatingAdjoint gradient of the
mean negative log-likelihood.

Tolerances: logpx 1e-4 relative to max|logpx| (adaptive FP32 vs FP64 at
1e-7); gradients 1e-3 relative (norm)."""
import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]


def _case(d, H, B, act, exact, seed, tol=1e-7):
    import gbnde
    from oracle import ffjord as off
    from oracle import mlp as omlp
    from oracle import tsit5 as ots
    rng = np.random.default_rng(seed)
    model = gbnde.Chain(gbnde.Dense(d + 1, H, act), gbnde.Dense(H, H, act), gbnde.Dense(H, d))
    p = model.init_params(rng)
    x = rng.standard_normal((d, B)).astype(np.float32)
    fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5(), abstol=tol, reltol=tol, time_input=True)
    noise = None if exact else fj.draw_noise(rng, B)
    logpx, zT, st = fj.forward_np(x, p, noise)
    assert st.retcode == 0
    om = omlp.MLP(model.dims, model.acts, time_input=True)
    rhs = off.FFJORDRHS(om, p.astype(np.float64), noise=None if exact else noise.T.astype(np.float64),
                        exact=exact)
    y0 = np.vstack([x.astype(np.float64), np.zeros((1, B))])
    ys, fwd = ots.solve_forward(rhs, y0, 0.0, 1.0, [1.0], tol, tol)
    ref = off.logpx_from_final(ys[..., 0], d)
    assert np.abs(logpx - ref).max() < 1e-4 * np.abs(ref).max()
    assert np.abs(zT - ys[:d, :, 0]).max() < 1e-4 * np.abs(ys[:d]).max()
    # gradient of the mean negative log-likelihood
    g = -np.ones(B) / B
    dx, dp, sta = fj.backward_np(g.astype(np.float32))
    assert sta.retcode_adj == 0
    dy = np.vstack([-ys[:d, :, 0] * g, -g[None, :]])
    gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, [1.0], dy[..., None], 0.0, tol, tol)
    rel = lambda a, b: np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)  # noqa: E731
    assert rel(dp, gp) < 1e-3
    assert rel(dx, gu[:d]) < 1e-3


@pytest.mark.parametrize("exact", [False, True])
def test_ffjord_small(exact):
    _case(2, 16, 64, "tanh", exact, 0)


def test_ffjord_config3_structure():
    """d = 16, (16+1) -> 512 -> 512 -> 16 softplus with time concatenated."""
    _case(16, 512, 96, "softplus", False, 1, tol=1e-5)


def test_ffjord_layer_torch_autograd():
    import torch

    import gbnde
    d, H, B = 2, 12, 32
    rng = np.random.default_rng(3)
    model = gbnde.Chain(gbnde.Dense(d + 1, H, "tanh"), gbnde.Dense(H, d))
    fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5(), abstol=1e-6, reltol=1e-6, time_input=True)
    p, st = fj.setup(rng)
    x = torch.tensor(rng.standard_normal((d, B)).astype(np.float32), requires_grad=True)
    pt = torch.tensor(p, requires_grad=True)
    (logpx, _, _), st = fj(x, pt, st)
    loss = -logpx.mean()
    loss.backward()
    assert torch.isfinite(pt.grad).all() and torch.count_nonzero(pt.grad) > 0
    assert x.grad.shape == x.shape and torch.isfinite(x.grad).all()


def test_ffjord_distribution_sampling_inverts_the_flow():
    """rand() solves the flow backwards (reverse tspan); pushing the samples
    forward again must return the base draws (src/ffjord.jl:183-246)."""
    import gbnde
    d, H, n = 2, 16, 64
    rng = np.random.default_rng(4)
    model = gbnde.Chain(gbnde.Dense(d + 1, H, "tanh"), gbnde.Dense(H, d))
    fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5(), abstol=1e-8, reltol=1e-8, time_input=True)
    p, st = fj.setup(rng)
    st["rng"] = np.random.default_rng(9)
    dist = gbnde.FFJORDDistribution(fj, p, st)
    z = dist.rand(n)
    assert z.shape == (d, n) and np.all(np.isfinite(z))
    base = np.random.default_rng(9).standard_normal((d, n)).astype(np.float32)
    _, zT, _ = fj.forward_np(z, p, fj.draw_noise(np.random.default_rng(1), n))
    assert np.abs(zT - base).max() < 1e-4 * max(1.0, np.abs(base).max())
    lp = dist.logpdf(z)
    assert lp.shape == (n,) and np.all(np.isfinite(lp))


def test_augmented_layer_pads_the_state():
    import gbnde
    S, a = 2, 2
    model = gbnde.Chain(gbnde.Dense(S + a, 8, "tanh"), gbnde.Dense(8, S + a))
    node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5(), saveat=[0.0, 1.0])
    anode = gbnde.AugmentedNDELayer(node, a)
    p, st = anode.setup(np.random.default_rng(0))
    x = np.array([[1.0, 0.5], [0.0, -0.5]], np.float32)
    sol, _ = anode(x, p, st)
    arr = np.asarray(sol)
    assert arr.shape == (S + a, 2, 2)
    assert np.allclose(arr[S:, :, 0], 0.0)


class _DiagNormal:
    """A diagonal Gaussian base density, logpdf(z) for z of shape (d, B)."""

    def __init__(self, mu, sig):
        self.mu, self.sig = mu, sig

    def logpdf(self, z):
        import torch
        if isinstance(z, torch.Tensor):
            mu = torch.as_tensor(self.mu, dtype=z.dtype, device=z.device)[:, None]
            sig = torch.as_tensor(self.sig, dtype=z.dtype, device=z.device)[:, None]
            return (-0.5 * ((z - mu) / sig) ** 2 - torch.log(sig) - 0.5 * np.log(2 * np.pi)).sum(0)
        mu, sig = self.mu[:, None], self.sig[:, None]
        return (-0.5 * ((z - mu) / sig) ** 2 - np.log(sig) - 0.5 * np.log(2 * np.pi)).sum(0)


def test_ffjord_user_basedist_value_and_gradient():
    """basedist = a diagonal Gaussian (src/ffjord.jl:170-176: logpdf(basedist, z)):
    logpx = logpdf(z(t1)) - delta_logp(t1) against the FP64 oracle's z(t1) and
    delta_logp (1e-4), and the gradient of the mean NLL against the oracle's
    adjoint with the cotangent dL/dz(t1) of the new base density (1e-3)."""
    import torch

    import gbnde
    from oracle import ffjord as off
    from oracle import mlp as omlp
    from oracle import tsit5 as ots
    d, H, B, tol = 2, 16, 48, 1e-7
    rng = np.random.default_rng(8)
    model = gbnde.Chain(gbnde.Dense(d + 1, H, "tanh"), gbnde.Dense(H, H, "tanh"), gbnde.Dense(H, d))
    base = _DiagNormal(np.array([0.3, -0.2]), np.array([0.7, 1.4]))
    fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5(), abstol=tol, reltol=tol, time_input=True,
                      basedist=base)
    p, st = fj.setup(rng)
    st["monte_carlo"] = False   # exact trace: deterministic
    x = rng.standard_normal((d, B)).astype(np.float32)
    pt = torch.tensor(p, requires_grad=True)
    (logpx, dlp, _), _ = fj(torch.tensor(x), pt, st)
    (-logpx.mean()).backward()
    om = omlp.MLP(model.dims, model.acts, time_input=True)
    rhs = off.FFJORDRHS(om, p.astype(np.float64), exact=True)
    y0 = np.vstack([x.astype(np.float64), np.zeros((1, B))])
    ys, fwd = ots.solve_forward(rhs, y0, 0.0, 1.0, [1.0], tol, tol)
    zT, delta = ys[:d, :, 0], ys[d, :, 0]
    ref = base.logpdf(zT) - delta
    assert np.abs(logpx.detach().numpy().ravel() - ref).max() < 1e-4 * np.abs(ref).max()
    assert np.abs(dlp.detach().numpy().ravel() - delta).max() < 1e-4 * max(1.0, np.abs(delta).max())
    # L = -mean(logpdf(z) - delta): dL/dz = -(dlogpdf/dz)/B, dL/ddelta = 1/B
    dz = ((zT - base.mu[:, None]) / base.sig[:, None] ** 2) / B
    dy = np.vstack([dz, np.full((1, B), 1.0 / B)])
    gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, [1.0], dy[..., None], 0.0, tol, tol)
    rel = np.linalg.norm(pt.grad.numpy() - gp) / np.linalg.norm(gp)
    assert rel < 1e-3, rel


def _case_bf16(d, H, B, act, seed, tol=1e-6):
    """FFJORD in the BF16 form: the stash engine's primal and tangent chains
    in the forward (Hutchinson), reverse-over-forward on the tensor cores in
    the adjoint. Against the FP64 oracle: logpx 1e-3 (relative to max|logpx|),
    z(t1) 1e-3, gradients of the mean NLL 1e-3 (relative norm)."""
    import gbnde
    from gbnde import _lib
    from oracle import ffjord as off
    from oracle import mlp as omlp
    from oracle import tsit5 as ots
    rng = np.random.default_rng(seed)
    model = gbnde.Chain(gbnde.Dense(d + 1, H, act), gbnde.Dense(H, H, act), gbnde.Dense(H, d))
    p = model.init_params(rng)
    x = rng.standard_normal((d, B)).astype(np.float32)
    fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5("bf16"), abstol=tol, reltol=tol, time_input=True)
    noise = fj.draw_noise(rng, B)
    logpx, zT, st = fj.forward_np(x, p, noise)
    assert st.retcode == 0
    assert st.fwd_path == _lib.PATH_TC
    om = omlp.MLP(model.dims, model.acts, time_input=True)
    rhs = off.FFJORDRHS(om, p.astype(np.float64), noise=noise.T.astype(np.float64), exact=False)
    y0 = np.vstack([x.astype(np.float64), np.zeros((1, B))])
    ys, fwd = ots.solve_forward(rhs, y0, 0.0, 1.0, [1.0], tol, tol)
    ref = off.logpx_from_final(ys[..., 0], d)
    assert np.abs(logpx - ref).max() < 1e-3 * np.abs(ref).max()
    assert np.abs(zT - ys[:d, :, 0]).max() < 1e-3 * np.abs(ys[:d]).max()
    g = -np.ones(B) / B
    dx, dp, sta = fj.backward_np(g.astype(np.float32))
    assert sta.retcode_adj == 0
    assert sta.adj_path == _lib.PATH_TC
    dy = np.vstack([-ys[:d, :, 0] * g, -g[None, :]])
    gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, [1.0], dy[..., None], 0.0, tol, tol)
    rel = lambda a, b: np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)  # noqa: E731
    assert rel(dp, gp) < 1e-3, rel(dp, gp)
    assert rel(dx, gu[:d]) < 1e-3, rel(dx, gu[:d])


def test_ffjord_bf16_small():
    _case_bf16(2, 32, 300, "tanh", 5)


def test_ffjord_bf16_config3_structure():
    """d = 16, (16+1) -> 512 -> 512 -> 16 softplus with time concatenated, on the tensor cores."""
    _case_bf16(16, 512, 256, "softplus", 6, tol=1e-5)


def _case_reg(d, H, B, act, exact, seed, wa, wb, precision="fp32", tol=1e-7):
    """regularize = true (src/ffjord.jl:131-132): the |f|^2 and |e^T J| rows
    against the FP64 oracle (values 1e-4 relative to their max), and the
    gradient of -mean(logpx) + wa mean(lambda1) + wb mean(lambda2) through the
    adjoint (1e-3 relative norm). Either precision runs the FP32 kernels."""
    import gbnde
    from gbnde import _lib
    from oracle import ffjord as off
    from oracle import mlp as omlp
    from oracle import tsit5 as ots
    rng = np.random.default_rng(seed)
    model = gbnde.Chain(gbnde.Dense(d + 1, H, act), gbnde.Dense(H, H, act), gbnde.Dense(H, d))
    p = model.init_params(rng)
    x = rng.standard_normal((d, B)).astype(np.float32)
    fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5(precision), abstol=tol, reltol=tol,
                      time_input=True, noise="gaussian")
    noise = fj.draw_noise(rng, B)
    logpx, zT, rf, rj, st = fj.forward_reg_np(x, p, noise, exact)
    assert st.retcode == 0 and st.fwd_path == _lib.PATH_FP32
    om = omlp.MLP(model.dims, model.acts, time_input=True)
    rhs = off.FFJORDRHS(om, p.astype(np.float64), noise=noise.T.astype(np.float64), exact=exact,
                        regularize=True)
    y0 = np.vstack([x.astype(np.float64), np.zeros((3, B))])
    ys, fwd = ots.solve_forward(rhs, y0, 0.0, 1.0, [1.0], tol, tol)
    yT = ys[..., 0]
    ref = off.logpx_from_final(yT, d)
    assert np.abs(logpx - ref).max() < 1e-4 * np.abs(ref).max()
    assert np.abs(zT - yT[:d]).max() < 1e-4 * np.abs(yT[:d]).max()
    assert np.abs(rf - yT[d + 1]).max() < 1e-4 * np.abs(yT[d + 1]).max()
    assert np.abs(rj - yT[d + 2]).max() < 1e-4 * np.abs(yT[d + 2]).max()
    g = -np.ones(B) / B
    drf = np.full(B, wa / B, np.float32)
    drj = np.full(B, wb / B, np.float32)
    dx, dp, sta = fj.backward_reg_np(g.astype(np.float32), None, drf, drj)
    assert sta.retcode_adj == 0 and sta.adj_path == _lib.PATH_FP32
    dy = np.vstack([-yT[:d] * g, -g[None, :], drf[None, :].astype(np.float64), drj[None, :].astype(np.float64)])
    gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, [1.0], dy[..., None], 0.0, tol, tol)
    rel = lambda a, b: np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)  # noqa: E731
    assert rel(dp, gp) < 1e-3, rel(dp, gp)
    assert rel(dx, gu[:d]) < 1e-3, rel(dx, gu[:d])


@pytest.mark.parametrize("exact", [False, True])
def test_ffjord_regularized_rows_and_gradient(exact):
    _case_reg(2, 16, 64, "tanh", exact, 11, 0.5, 0.8)


def test_ffjord_regularized_without_the_ej_cotangent():
    """lambda2 unused in the loss (the reference's tests): the |e^T J| pass of
    the adjoint is skipped, the |f|^2 term still enters."""
    _case_reg(2, 16, 64, "softplus", False, 12, 0.3, 0.0)


def test_ffjord_regularized_config3_structure_bf16_request():
    """d = 16, (16+1) -> 512 -> 512 -> 16 softplus, BF16 requested: the
    regularised system runs on the FP32 kernels and the stats say so."""
    _case_reg(16, 512, 96, "softplus", False, 13, 0.1, 0.1, precision="bf16", tol=1e-5)


def test_ffjord_regularized_layer_torch_autograd():
    """(logpx, lambda1, lambda2) from the layer with st regularize = true; the
    gradient of a loss using all three matches the C-ABI backward."""
    import torch

    import gbnde
    d, H, B = 2, 12, 32
    rng = np.random.default_rng(14)
    model = gbnde.Chain(gbnde.Dense(d + 1, H, "tanh"), gbnde.Dense(H, d))
    fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5(), abstol=1e-6, reltol=1e-6, time_input=True)
    p, st = fj.setup(rng)
    st["regularize"] = True
    st["rng"] = np.random.default_rng(5)
    x = rng.standard_normal((d, B)).astype(np.float32)
    pt = torch.tensor(p, requires_grad=True)
    (logpx, l1, l2), _ = fj(torch.tensor(x), pt, st)
    assert logpx.shape == (1, B) and l1.shape == (1, B) and l2.shape == (1, B)
    assert torch.all(l1 > 0) and torch.all(l2 > 0)
    loss = -logpx.mean() + 0.1 * l1.mean() + 0.2 * l2.mean()
    loss.backward()
    noise = fj.draw_noise(np.random.default_rng(5), B)
    lp2, _, rf, rj, _ = fj.forward_reg_np(x, p, noise, False)
    assert np.allclose(lp2, logpx.detach().numpy().ravel()) and np.allclose(rf, l1.detach().numpy().ravel())
    _, dp, _ = fj.backward_reg_np(np.full(B, -1.0 / B, np.float32), None, np.full(B, 0.1 / B, np.float32),
                                  np.full(B, 0.2 / B, np.float32))
    assert np.allclose(pt.grad.numpy(), dp, rtol=1e-5, atol=1e-7)


def test_ffjord_distribution_sampling_with_the_regulariser_rows():
    """rand() with st regularize = true solves the reversed flow with the two
    regulariser rows riding along (src/ffjord.jl:192-213); pushing the
    samples forward through the regularised system returns the base draws."""
    import gbnde
    d, H, n = 2, 16, 64
    rng = np.random.default_rng(15)
    model = gbnde.Chain(gbnde.Dense(d + 1, H, "tanh"), gbnde.Dense(H, d))
    fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5(), abstol=1e-8, reltol=1e-8, time_input=True)
    p, st = fj.setup(rng)
    st["regularize"] = True
    st["rng"] = np.random.default_rng(9)
    dist = gbnde.FFJORDDistribution(fj, p, st)
    z = dist.rand(n)
    assert z.shape == (d, n) and np.all(np.isfinite(z))
    base = np.random.default_rng(9).standard_normal((d, n)).astype(np.float32)
    _, zT, rf, rj, _ = fj.forward_reg_np(z, p, fj.draw_noise(np.random.default_rng(1), n), False)
    assert np.abs(zT - base).max() < 1e-4 * max(1.0, np.abs(base).max())
    assert np.all(rf > 0) and np.all(rj > 0)
