"""CPU checks of host-side logic: the Float32-time selection of the layers
and the descriptors they build, and the bench's synthetic workloads (Glorot
parameters in the flat ComponentArray layout, targets of the random stable
linear ODE). No GPU and no library load."""
import numpy as np
import pytest


def test_float32_time_follows_a_float32_tspan():
    import gbnde
    from gbnde import _lib
    model = gbnde.Chain(gbnde.Dense(2, 8, "tanh"), gbnde.Dense(8, 2))
    ts = np.linspace(0.0, 1.5, 7)
    n32 = gbnde.NeuralODE(model, (np.float32(0.0), np.float32(1.5)), gbnde.Tsit5("fp32"), saveat=ts)
    assert n32.float32_time
    d = n32.desc()
    assert d.flags == _lib.FLAG_FP32_TIME
    # save points become Float32 values
    assert all(float(np.float32(s)) == s for s in n32.saveat)
    n64 = gbnde.NeuralODE(model, (0.0, 1.5), gbnde.Tsit5("fp32"), saveat=ts)
    assert not n64.float32_time and n64.desc().flags == 0
    # the BF16 form keeps FP64 time: not chosen automatically, refused when asked for
    nb = gbnde.NeuralODE(model, (np.float32(0.0), np.float32(1.5)), gbnde.Tsit5("bf16"), saveat=ts)
    assert not nb.float32_time
    with pytest.raises(ValueError):
        gbnde.NeuralODE(model, (0.0, 1.5), gbnde.Tsit5("bf16"), saveat=ts, float32_time=True)


def test_glorot_parameters_layout():
    import bench
    rng = np.random.default_rng(0)
    dims = [3, 5, 4]
    p = bench.glorot_params(dims, rng)
    assert p.dtype == np.float32 and p.size == 3 * 5 + 5 + 5 * 4 + 4
    off = 0
    for i in range(len(dims) - 1):
        n_w = dims[i] * dims[i + 1]
        lim = np.sqrt(6.0 / (dims[i] + dims[i + 1]))
        assert np.all(np.abs(p[off:off + n_w]) <= lim)
        off += n_w
        assert np.all(p[off:off + dims[i + 1]] == 0.0)  # zero biases
        off += dims[i + 1]


def test_sweep_targets_solve_the_linear_ode():
    import torch

    import bench
    dims, p, ts, u0, tg, E = bench.sweep_data(4, 8, 16, torch.device("cpu"))
    assert tuple(tg.shape) == (len(ts), 16, 4)
    # t = 0: the initial state; and every target is exp(M t_k) applied to u0
    assert torch.allclose(tg[0], u0, atol=1e-6)
    for k in (3, len(ts) - 1):
        assert torch.allclose(tg[k], u0 @ E[k].T, atol=1e-5)
    # M is stable (eigenvalues in [-2, -0.1]): the targets shrink
    assert float(tg[-1].norm()) < float(tg[0].norm())
