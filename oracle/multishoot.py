"""FP64 restatement of DiffEqFlux's multiple shooting (test infrastructure only).

Follows src/multiple_shooting.jl: `group_ranges` (:231-239) cuts the save grid
into overlapping ranges i:min(n, i+gs-1) for i in 1:gs-1:n-1; every range is
solved on its own from the data point at its first time (:52-62); the loss is
the sum of the user loss over the groups plus continuity_term * sum(abs,
pred_prev_end - data_first) for consecutive groups (:70-81, :243); any failed
solve makes the loss Inf (:66-67). Ranges here are 0-based (start, stop)
with stop inclusive.
"""
import numpy as np

try:
    from . import tsit5 as ots
except ImportError:  # pragma: no cover
    import tsit5 as ots  # type: ignore


def group_ranges(datasize, groupsize):
    if not (2 <= groupsize <= datasize):
        raise ValueError("groupsize must be within [2, datasize]")
    return [(i, min(datasize - 1, i + groupsize - 1)) for i in range(0, datasize - 1, groupsize - 1)]


def solve_groups(rhs, data, tsteps, groupsize, abstol, reltol):
    """data: S x datasize. Returns (list of S x len(range) predictions, all_ok)."""
    preds, ok = [], True
    for (a, b) in group_ranges(data.shape[1], groupsize):
        ts = tsteps[a:b + 1]
        us, integ = ots.solve_forward(rhs, data[:, a:a + 1], ts[0], ts[-1], ts, abstol, reltol)
        ok = ok and integ.retcode == ots.RET_SUCCESS
        preds.append(us[:, 0, :])
    return preds, ok


def multiple_shoot_loss(preds, data, groupsize, continuity_term=100.0, loss_fn=None):
    """Loss of src/multiple_shooting.jl:70-81 with the default continuity loss."""
    if loss_fn is None:
        loss_fn = lambda u, uh: float(np.sum((u - uh) ** 2))  # noqa: E731
    loss = 0.0
    rngs = group_ranges(data.shape[1], groupsize)
    for i, (a, b) in enumerate(rngs):
        u = data[:, a:b + 1]
        loss += loss_fn(u, preds[i])
        if i > 0:
            loss += continuity_term * float(np.sum(np.abs(preds[i - 1][:, -1] - u[:, 0])))
    return loss
