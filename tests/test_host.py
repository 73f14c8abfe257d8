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


def test_multishoot_packing_matches_per_trajectory_slices():
    """The packed initial states and save-point data of many trajectories
    (rows of the concatenated data, gathered through the cached layout) equal
    each trajectory's own group slices (src/multiple_shooting.jl:52-62,
    group_ranges at :231-239); data whose length disagrees with its times is
    rejected."""
    import pytest

    from gbnde import multiple_shooting as ms
    rng = np.random.default_rng(7)
    S = 5
    trajs = []
    for _ in range(9):
        n = int(rng.integers(6, 30))
        trajs.append((rng.standard_normal((S, n)).astype(np.float32), 0.1 * np.arange(n), int(rng.integers(2, 7))))
    P = ms._Packed(trajs)
    u0, data = [], []
    for d, ts, gs in trajs:
        for rg in ms.group_ranges(len(ts), gs):
            u0.append(d[:, rg.start])
            data.extend(d[:, k] for k in rg)
    assert np.array_equal(P.u0, np.array(u0)) and np.array_equal(P.data, np.array(data))
    assert P.u0.flags.c_contiguous and P.data.flags.c_contiguous
    assert P.nseg == len(u0) and len(P.saveat) == len(data)
    bad = list(trajs)
    bad[3] = (bad[3][0][:, :-1], bad[3][1], bad[3][2])
    with pytest.raises(ValueError):
        ms._Packed(bad)


def test_multishoot_layout_cache_follows_the_times():
    """A cached segment table is reused only for the same times: trajectories
    with the same lengths, group sizes and end points but other interior
    times get their own save times."""
    from gbnde import multiple_shooting as ms
    d = np.zeros((2, 7), np.float32)
    t1 = np.linspace(0.0, 1.0, 7)
    t2 = t1.copy()
    t2[3] = 0.55
    a = ms._Packed([(d, t1, 3)])
    b = ms._Packed([(d, t2, 3)])
    c = ms._Packed([(d, t1, 3)])
    assert np.array_equal(a.saveat[[0, 1, 2]], t1[:3]) and 0.55 in b.saveat and 0.55 not in c.saveat
