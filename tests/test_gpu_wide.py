"""BF16 tensor-core form in stash mode (fwd_tcw / bwd_tcw: state up to 256,
widths up to 1024, an optional time row) against the FP64 oracle, through
the C ABI.

Tolerances (relative), as for the single-accumulator kernels:
  * saved states vs the oracle replaying the kernel's accepted steps: 2e-5
  * loss and gradient vs the free-running FP64 oracle: 1e-3
"""
import numpy as np
import pytest

from conftest import gpu_available
from test_gpu_neural_ode import _rel

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]

CASES = {
    # id: (S, H, act, B, time_input)
    "s64_h512": (64, 512, "tanh", 200, False),
    "s256_h128": (256, 128, "tanh", 130, False),
    "s16_h1024": (16, 1024, "tanh", 64, False),
    "s16_h512_softplus_time": (16, 512, "softplus", 96, True),
}


def _model(S, H, act, tin, seed):
    import gbnde
    rng = np.random.default_rng(seed)
    model = gbnde.Chain(gbnde.Dense(S + (1 if tin else 0), H, act), gbnde.Dense(H, H, act), gbnde.Dense(H, S))
    p = model.init_params(rng)
    dims = model.dims
    off = 0
    for i in range(3):
        off += dims[i] * dims[i + 1]
        p[off:off + dims[i + 1]] = 0.02 * rng.standard_normal(dims[i + 1])
        off += dims[i + 1]
    return model, p, rng


@pytest.mark.parametrize("case", list(CASES))
def test_wide_forward_and_gradient_vs_oracle(case):
    import gbnde
    from gbnde import _lib
    from oracle import mlp as omlp
    from oracle import tsit5 as ots
    S, H, act, B, tin = CASES[case]
    model, p, rng = _model(S, H, act, tin, 7)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    ts = np.linspace(0.0, 1.0, 8)
    tol = (1e-7, 1e-5)
    s = gbnde.Solver(model, "bf16", 0, time_input=tin)
    desc = gbnde.Solver.solve_desc(0.0, 1.0, ts, tol[0], tol[1], 0)
    s.set_params(p)
    us, st = s.forward(u0, desc)
    assert st.retcode == 0
    assert st.fwd_path == _lib.PATH_TC
    om = omlp.MLP(model.dims, model.acts, time_input=tin)
    rhs = omlp.MLPRHS(om, p.astype(np.float64))
    steps = s.forward_steps()
    ous, _ = ots.solve_forward(rhs, u0.astype(np.float64), 0.0, 1.0, ts, tol[0], tol[1], steps=steps)
    assert _rel(us, ous) < 2e-5, _rel(us, ous)
    ous2, fwd2 = ots.solve_forward(omlp.MLPRHS(om, p.astype(np.float64)), u0.astype(np.float64), 0.0, 1.0, ts,
                                   tol[0], tol[1])
    tgt = 0.5 * np.random.default_rng(1).standard_normal(ous2.shape)
    L64 = np.mean((ous2 - tgt) ** 2)
    L = np.mean((us.astype(np.float64) - tgt) ** 2)
    assert abs(L - L64) / L64 < 1e-3
    g = (2.0 * (us.astype(np.float64) - tgt) / us.size).astype(np.float32)
    du0, dp, sta = s.backward(g)
    assert sta.retcode_adj == 0
    assert sta.adj_path == _lib.PATH_TC
    gu, gp, _ = ots.adjoint_interpolating(omlp.MLPRHS(om, p.astype(np.float64)), fwd2, ts,
                                          2.0 * (ous2 - tgt) / ous2.size, 0.0, tol[0], tol[1])
    assert _rel(du0, gu) < 1e-3, _rel(du0, gu)
    assert _rel(dp, gp) < 1e-3, _rel(dp, gp)
    assert st.naccept + st.nreject <= 3 * (fwd2.naccept + fwd2.nreject) + 4
    s.close()
