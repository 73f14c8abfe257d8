"""CPU checks of the FP64 oracle (no GPU): the Tsit5 tableau pin, known-answer
solutions, agreement with an independent integrator, adjoint gradients
against finite differences and against torch autograd, and reproduction of the
committed golden fixtures."""
import os

import numpy as np
import pytest

from oracle import check_tableau
from oracle import mlp as omlp
from oracle import tsit5 as ots

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_tableau_order_conditions():
    r = check_tableau.residuals()
    assert r["row_sum"] < 1e-14
    assert r["b_order5"] < 1e-13
    assert r["bhat_order4"] < 1e-13
    assert r["bhat_not_order5"] > 1e-6          # the embedded pair really differs
    assert r["dense_order4"] < 1e-12
    assert r["dense_at_1_equals_b"] < 1e-13


def test_linear_ode_known_answer():
    from scipy.linalg import expm
    rng = np.random.default_rng(0)
    S, B = 5, 3
    Q, _ = np.linalg.qr(rng.standard_normal((S, S)))
    M = Q @ np.diag(-rng.uniform(0.1, 2.0, S)) @ Q.T

    class Lin:
        def f(self, u, t):
            return M @ u

    u0 = rng.standard_normal((S, B))
    ts = np.linspace(0, 1, 11)
    us, integ = ots.solve_forward(Lin(), u0, 0.0, 1.0, ts, 1e-10, 1e-10)
    exact = np.stack([expm(M * t) @ u0 for t in ts], -1)
    assert np.abs(us - exact).max() < 1e-9
    assert integ.retcode == ots.RET_SUCCESS and integ.nreject >= 0


def test_spiral_against_dop853():
    from scipy.integrate import solve_ivp
    A = np.array([[-0.1, 2.0], [-2.0, -0.1]])

    class Sp:
        def f(self, u, t):
            return ((u ** 3).T @ A).T

    ts = np.linspace(0, 1.5, 30)
    us, _ = ots.solve_forward(Sp(), np.array([[2.0], [0.0]]), 0.0, 1.5, ts, 1e-12, 1e-12)
    ref = solve_ivp(lambda t, u: (u ** 3) @ A, (0, 1.5), [2.0, 0.0], method="DOP853", rtol=1e-13,
                    atol=1e-13, t_eval=ts)
    assert np.abs(us[:, 0, :] - ref.y).max() < 1e-10


def test_step_size_controller_behaviour():
    """Looser tolerances take fewer steps; clipping lands exactly on t1; the
    evaluation count is 1 (f(u0), shared by the initial-step algorithm and the
    first FSAL stage) + 1 (initial-step probe) + 6 per attempted step."""
    m = omlp.MLP([2, 16, 2], ["tanh", "identity"], cube_input=True)
    p = m.glorot_uniform(np.random.default_rng(3)).astype(np.float64)
    u0 = np.array([[2.0], [0.0]])
    counts = []
    for tol in (1e-4, 1e-6, 1e-8):
        rhs = omlp.MLPRHS(m, p)
        _, integ = ots.solve_forward(rhs, u0, 0.0, 1.5, [1.5], tol, tol)
        counts.append(integ.naccept)
        assert integ.t == 1.5
        assert rhs.nf == 2 + 6 * (integ.naccept + integ.nreject)
    assert counts[0] <= counts[1] <= counts[2]


@pytest.mark.parametrize("sense", ["interpolating", "backsolve", "gauss"])
def test_adjoint_matches_finite_differences(sense):
    rng = np.random.default_rng(1)
    m = omlp.MLP([2, 12, 2], ["tanh", "identity"], cube_input=True)
    p = m.glorot_uniform(rng).astype(np.float64)
    p[-2:] = 0.1
    u0 = np.array([[1.5, 0.5], [0.0, -0.5]])
    ts = np.linspace(0, 1.0, 8)
    tgt = 0.3 * rng.standard_normal((2, 2, 8))
    tol = 1e-10

    def loss(pp, uu):
        us, _ = ots.solve_forward(omlp.MLPRHS(m, pp), uu, 0.0, 1.0, ts, tol, tol)
        return np.sum((us - tgt) ** 2)

    rhs = omlp.MLPRHS(m, p)
    us, fwd = ots.solve_forward(rhs, u0, 0.0, 1.0, ts, tol, tol)
    dL = 2 * (us - tgt)
    if sense == "interpolating":
        gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, ts, dL, 0.0, tol, tol)
    elif sense == "gauss":
        gu, gp, _ = ots.adjoint_gauss(rhs, fwd, ts, dL, 0.0, tol, tol)
    else:
        gu, gp, _ = ots.adjoint_backsolve(rhs, us, ts, dL, 0.0, tol, tol)
    eps = 1e-6
    fdp = np.array([(loss(p + eps * e, u0) - loss(p - eps * e, u0)) / (2 * eps) for e in np.eye(p.size)])
    fdu = np.zeros_like(u0)
    for i in np.ndindex(u0.shape):
        e = np.zeros_like(u0)
        e[i] = eps
        fdu[i] = (loss(p, u0 + e) - loss(p, u0 - e)) / (2 * eps)
    assert np.linalg.norm(gp - fdp) / np.linalg.norm(fdp) < 1e-6
    assert np.linalg.norm(gu - fdu) / np.linalg.norm(fdu) < 1e-6


def test_mlp_vjp_against_torch_autograd():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    for acts, cube in ((["tanh", "tanh", "identity"], False), (["softplus", "identity"], True)):
        dims = [4, 7, 7, 4] if len(acts) == 3 else [4, 9, 4]
        m = omlp.MLP(dims, acts, cube_input=cube)
        p = rng.standard_normal(m.nparams())
        u = rng.standard_normal((4, 5))
        lam = rng.standard_normal((4, 5))
        gu, gp = m.vjp(p, u, 0.0, lam)
        pt = torch.tensor(p, requires_grad=True)
        ut = torch.tensor(u, requires_grad=True)
        x = ut ** 3 if cube else ut
        o = 0
        for l, a in enumerate(acts):
            din, dout = dims[l], dims[l + 1]
            W = pt[o:o + din * dout].reshape(din, dout).T
            o += din * dout
            b = pt[o:o + dout]
            o += dout
            x = W @ x + b[:, None]
            x = torch.tanh(x) if a == "tanh" else (torch.nn.functional.softplus(x) if a == "softplus" else x)
        (x * torch.tensor(lam)).sum().backward()
        assert np.allclose(gu, ut.grad.numpy(), rtol=1e-12, atol=1e-12)
        assert np.allclose(gp, pt.grad.numpy(), rtol=1e-12, atol=1e-12)


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


@pytest.mark.parametrize("name", ["spiral.npz", "batched.npz"])
def test_oracle_reproduces_golden_fixtures(name):
    g = _load(name)
    dims = [int(d) for d in g["dims"]]
    acts = ["tanh"] * (len(dims) - 2) + ["identity"]
    m = omlp.MLP(dims, acts, cube_input=bool(g["cube"]))
    rhs = omlp.MLPRHS(m, g["p"].astype(np.float64))
    us, fwd = ots.solve_forward(rhs, g["u0"], 0.0, float(g["ts"][-1]), g["ts"], float(g["abstol"]),
                                float(g["reltol"]))
    assert np.array_equal(us, g["usave"])
    assert fwd.naccept == int(g["naccept"])
    gu, gp, _ = ots.adjoint_interpolating(rhs, fwd, g["ts"], g["dLdu"], 0.0, float(g["abstol"]),
                                          float(g["reltol"]))
    assert np.array_equal(gu, g["gu_interp"]) and np.array_equal(gp, g["gp_interp"])
    # the two adjoints agree to the solver tolerance
    assert np.linalg.norm(g["gp_back"] - g["gp_interp"]) / np.linalg.norm(g["gp_interp"]) < 1e-3


def test_linear_fixture_is_the_exact_solution():
    g = _load("linear.npz")
    assert np.abs(g["usave"] - g["exact"]).max() < 1e-8


def test_float32_time_mode_keeps_float32_times():
    """The oracle's Float32-time mode: accepted step times and sizes are Float32
    values, and the solution agrees with the FP64-time solve to the tolerance."""
    from oracle import mlp as omlp
    from oracle import tsit5 as ots
    rng = np.random.default_rng(2)
    om = omlp.MLP([2, 16, 2], ["tanh", "identity"], cube_input=True)
    P = om.nparams()
    rhs = omlp.MLPRHS(om, 0.3 * rng.standard_normal(P))
    u0 = np.array([[2.0], [0.0]])
    ts = np.linspace(0.0, 1.5, 10, dtype=np.float32).astype(np.float64)
    a, ia = ots.solve_forward(rhs, u0, 0.0, 1.5, ts, 1e-7, 1e-5, time_f32=True)
    b, ib = ots.solve_forward(rhs, u0, 0.0, 1.5, ts, 1e-7, 1e-5)
    for tn, h in ia.steps:
        assert float(np.float32(tn)) == tn and float(np.float32(h)) == abs(h)
    assert np.abs(a - b).max() < 1e-5 * np.abs(b).max()


@pytest.mark.parametrize("sense", ["interpolating", "backsolve", "gauss"])
def test_adjoint_linear_known_answer(sense):
    """The adjoints against closed forms on du/dt = M u with
    L = sum_k g_k . u(t_k): dL/du0 = sum_k exp(M t_k)^T g_k exactly, and dL/dM
    against central differences of the matrix-exponential solution (no
    integrator in the reference values)."""
    from scipy.linalg import expm
    rng = np.random.default_rng(5)
    S, B = 3, 2
    Q, _ = np.linalg.qr(rng.standard_normal((S, S)))
    M = Q @ np.diag(-rng.uniform(0.2, 1.5, S)) @ Q.T + 0.3 * rng.standard_normal((S, S))

    class Lin:
        def __init__(self, M):
            self.M = M

        def f(self, u, t):
            return self.M @ u

        def vjp(self, u, t, lam):
            return self.M.T @ lam, (lam @ u.T).reshape(-1)

        def nparams(self):
            return S * S

    u0 = rng.standard_normal((S, B))
    ts = np.linspace(0.0, 1.0, 6)
    g = rng.standard_normal((S, B, len(ts)))
    us, fwd = ots.solve_forward(Lin(M), u0, 0.0, 1.0, ts, 1e-12, 1e-12)
    if sense == "interpolating":
        gu, gp, _ = ots.adjoint_interpolating(Lin(M), fwd, ts, g, 0.0, 1e-12, 1e-12)
    elif sense == "backsolve":
        gu, gp, _ = ots.adjoint_backsolve(Lin(M), us, ts, g, 0.0, 1e-12, 1e-12)
    else:
        gu, gp, _ = ots.adjoint_gauss(Lin(M), fwd, ts, g, 0.0, 1e-12, 1e-12)
    exact_u0 = sum(expm(M * t).T @ g[..., k] for k, t in enumerate(ts))
    assert np.abs(gu - exact_u0).max() < 1e-8 * np.abs(exact_u0).max()

    def loss(Mx):
        return sum(float(np.sum(g[..., k] * (expm(Mx * t) @ u0))) for k, t in enumerate(ts))
    eps = 1e-6
    fd = np.zeros(S * S)
    for j in range(S * S):
        E = np.zeros(S * S)
        E[j] = eps
        fd[j] = (loss(M + E.reshape(S, S)) - loss(M - E.reshape(S, S))) / (2 * eps)
    assert np.abs(gp - fd).max() < 1e-6 * np.abs(fd).max()


def test_oracle_reproduces_the_ffjord_and_multishoot_fixtures():
    """ffjord.npz (exact trace) and multishoot.npz recomputed by the oracle:
    logpx, z(t1) and the step count; the group predictions and the loss."""
    from oracle import ffjord as off
    from oracle import multishoot as oms
    f = _load("ffjord.npz")
    dims = [int(x) for x in f["dims"]]
    d, B = dims[0], f["x"].shape[1]
    m = omlp.MLP(dims, ["tanh", "identity"])
    rhs = off.FFJORDRHS(m, f["p"].astype(np.float64), exact=True)
    ys, fwd = ots.solve_forward(rhs, np.vstack([f["x"], np.zeros((1, B))]), 0.0, 1.0, [1.0],
                                float(f["abstol"]), float(f["reltol"]))
    assert np.array_equal(off.logpx_from_final(ys[..., 0], d), f["logpx"])
    assert np.array_equal(ys[:d, :, 0], f["zT"]) and fwd.naccept == int(f["naccept"])
    g = _load("multishoot.npz")
    m2 = omlp.MLP([int(x) for x in g["dims"]], ["tanh", "identity"])
    preds, ok = oms.solve_groups(omlp.MLPRHS(m2, g["p"].astype(np.float64)), g["data"], g["ts"],
                                 int(g["group_size"]), float(g["abstol"]), float(g["reltol"]))
    assert ok and np.array_equal(np.concatenate(preds, axis=1), g["preds"])
    assert oms.multiple_shoot_loss(preds, g["data"], int(g["group_size"]), float(g["continuity_term"])) == g["loss"]
