"""Host-side mirror of DiffEqFlux's `multiple_shoot` on the packed GB300 kernel.

`multiple_shoot(p, ode_data, tsteps, model, loss_function, group_size;
continuity_term=100)` keeps the reference's signature and result
(`(loss, group_predictions)`, src/multiple_shooting.jl:36-94): the data grid
is cut by `group_ranges` (:231-239), every group is solved from its first data
point with its own adaptive controller, and the loss adds
continuity_term * continuity_loss(pred_prev_end, data_first). All groups -- of
one trajectory or, with `multiple_shoot_batch`, of many trajectories with
uneven lengths and group sizes -- run in one kernel launch. With torch tensors
for `p` the predictions are differentiable; their backward is the kernel's
discrete adjoint.
"""
import ctypes as C
import math

import numpy as np

from . import _lib


def group_ranges(datasize, groupsize):
    """0-based ranges of src/multiple_shooting.jl:231-239 (stop exclusive)."""
    if not (2 <= groupsize <= datasize):
        raise ValueError(f"groupsize must be within [2, datasize]; got {groupsize} for {datasize}")
    return [range(i, min(datasize, i + groupsize)) for i in range(0, datasize - 1, groupsize - 1)]


def _default_continuity_loss(u_end, u_0):
    return (u_end - u_0).abs().sum() if hasattr(u_end, "abs") else np.sum(np.abs(u_end - u_0))


class _Packed:
    """Segment table of one or many trajectories."""

    def __init__(self, trajectories):
        # trajectories: list of (data S x n, tsteps n, group_size)
        segs, saveat, u0, self.groups = [], [], [], []
        for ti, (data, ts, gs) in enumerate(trajectories):
            ts = np.asarray(ts, dtype=np.float64)
            for rg in group_ranges(len(ts), gs):
                seg = _lib.Segment()
                seg.t0, seg.t1 = float(ts[rg.start]), float(ts[rg.stop - 1])
                seg.save_off = len(saveat)
                seg.nsave = len(rg)
                segs.append(seg)
                saveat.extend(ts[rg.start:rg.stop].tolist())
                u0.append(np.asarray(data, dtype=np.float32)[:, rg.start])
                self.groups.append((ti, rg))
        self.segs = (_lib.Segment * len(segs))(*segs)
        self.saveat = np.ascontiguousarray(saveat, dtype=np.float64)
        self.u0 = np.ascontiguousarray(np.stack(u0, axis=1).T)  # nseg x S (column-major S x nseg)
        self.nseg = len(segs)


class MultipleShooter:
    """Packed forward and discrete-adjoint backward of multiple-shooting groups."""

    def __init__(self, solver, abstol=1e-6, reltol=1e-3, maxiters=100000):
        self.solver = solver
        self.abstol, self.reltol, self.maxiters = float(abstol), float(reltol), int(maxiters)

    def forward(self, packed, p):
        s = self.solver
        s.set_params(p)
        S = s.state_dim
        out = np.empty((len(packed.saveat), S), dtype=np.float32)
        ret = np.zeros(packed.nseg, dtype=np.int32)
        st = _lib.Stats()
        s.bump()
        _lib.check(s.lib.gbnde_multishoot_forward(
            s.h, S, packed.nseg, packed.segs, packed.saveat.ctypes.data_as(C.POINTER(C.c_double)),
            len(packed.saveat), packed.u0.ctypes.data, self.abstol, self.reltol, self.maxiters,
            out.ctypes.data, ret.ctypes.data_as(C.POINTER(C.c_int)), C.byref(st)))
        return out.T, ret, st  # S x nsave_total

    def backward(self, dL_dusave):
        s = self.solver
        g = np.ascontiguousarray(np.asarray(dL_dusave, dtype=np.float32).T)
        nseg = self._nseg
        du0 = np.empty((nseg, s.state_dim), dtype=np.float32)
        dp = np.empty(s.nparams, dtype=np.float32)
        st = _lib.Stats()
        _lib.check(s.lib.gbnde_multishoot_backward(s.h, g.ctypes.data, du0.ctypes.data, dp.ctypes.data,
                                                   C.byref(st)))
        return du0.T, dp


def _predict(shooter, packed, p):
    """Saved states (S x nsave_total); differentiable in p when p is a torch tensor."""
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(p, torch.Tensor):
        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, pt):
                us, ret, st = shooter.forward(packed, pt.detach().cpu().numpy())
                shooter._nseg = packed.nseg
                ctx.ret = ret
                return torch.from_numpy(np.ascontiguousarray(us)).to(pt.device), torch.from_numpy(ret)

            @staticmethod
            def backward(ctx, g, _gret):
                if np.any(ctx.ret != 0):
                    raise RuntimeError("cannot differentiate multiple shooting with a failed group")
                _, dp = shooter.backward(g.detach().cpu().numpy())
                return torch.from_numpy(dp).to(g.device)

        us, ret = _Fn.apply(p)
        return us, ret.numpy()
    us, ret, st = shooter.forward(packed, p)
    shooter._nseg = packed.nseg
    return us, ret


def _loss(packed, us, trajectories, loss_function, continuity_loss, continuity_term):
    loss = 0.0
    preds = []
    prev = None
    for k, (ti, rg) in enumerate(packed.groups):
        seg = packed.segs[k]
        pred = us[:, seg.save_off:seg.save_off + seg.nsave]
        data = trajectories[ti][0]
        u = data[:, rg.start:rg.stop]
        if hasattr(pred, "new_tensor") and not hasattr(u, "new_tensor"):
            u = pred.new_tensor(np.asarray(u, dtype=np.float32))
        loss = loss + loss_function(u, pred)
        if prev is not None and prev[0] == ti:
            loss = loss + continuity_term * continuity_loss(prev[1][:, -1], u[:, 0])
        prev = (ti, pred)
        preds.append(pred)
    return loss, preds


def multiple_shoot(p, ode_data, tsteps, model_or_solver, loss_function, group_size, *,
                   continuity_term=100.0, continuity_loss=None, abstol=1e-6, reltol=1e-3,
                   maxiters=100000, precision="fp32", device=0):
    """``multiple_shoot(p, ode_data, tsteps, model, loss, group_size; continuity_term=100)``.

    Returns ``(loss, group_predictions)``; the loss is ``inf`` when any group
    fails to solve (src/multiple_shooting.jl:66-67)."""
    return multiple_shoot_batch(p, [(ode_data, tsteps, group_size)], model_or_solver, loss_function,
                                continuity_term=continuity_term, continuity_loss=continuity_loss,
                                abstol=abstol, reltol=reltol, maxiters=maxiters, precision=precision,
                                device=device)


def multiple_shoot_batch(p, trajectories, model_or_solver, loss_function, *, continuity_term=100.0,
                         continuity_loss=None, abstol=1e-6, reltol=1e-3, maxiters=100000,
                         precision="fp32", device=0):
    """Many trajectories (data S x n_i, tsteps n_i, group_size_i), all groups in one launch.
    The loss sums the per-trajectory multiple-shooting losses."""
    from .layers import Chain, Solver
    solver = model_or_solver if isinstance(model_or_solver, Solver) else Solver(model_or_solver, precision, device)
    if continuity_loss is None:
        continuity_loss = _default_continuity_loss
    packed = _Packed(trajectories)
    shooter = MultipleShooter(solver, abstol, reltol, maxiters)
    us, ret = _predict(shooter, packed, p)
    preds_loss, preds = _loss(packed, us, trajectories, loss_function, continuity_loss, continuity_term)
    if np.any(ret != 0):
        return math.inf, preds
    return preds_loss, preds
