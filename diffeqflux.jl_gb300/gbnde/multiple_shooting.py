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
discrete adjoint. With `loss_function` = `mse_loss` / `sse_loss` (or "mse" /
"sse") and the default continuity loss, the loss and its cotangent are one
device kernel (gbnde_multishoot_loss) and the gradient runs from that
cotangent without a host round trip; any other loss function runs on the
host in torch/numpy, per group, as the reference's loop does.
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


def sse_loss(u, uh):
    """``sum(abs2, u .- uh)``: recognised by multiple_shoot, which then evaluates
    the whole loss (and the continuity terms) in one kernel on the device."""
    return ((u - uh) ** 2).sum()


def mse_loss(u, uh):
    """``mean(abs2, u .- uh)`` per group; the device-fused form, as sse_loss."""
    return ((u - uh) ** 2).mean()


_FUSED_KIND = {sse_loss: 0, mse_loss: 1, "sse": 0, "mse": 1}


class _Layout:
    """Segment table of a set of trajectories (lengths and group sizes): the
    packed save times, each trajectory's packed column indices into its data,
    the first data column of every segment and each segment's successor."""

    def __init__(self, shapes):
        segs, saveat, self.groups, self.cols, self.starts, nxt = [], [], [], [], [], []
        for ti, (ts, gs) in enumerate(shapes):
            ts = np.asarray(ts, dtype=np.float64)
            rgs = group_ranges(len(ts), gs)
            idx = []
            for k, rg in enumerate(rgs):
                seg = _lib.Segment()
                seg.t0, seg.t1 = float(ts[rg.start]), float(ts[rg.stop - 1])
                seg.save_off = len(saveat)
                seg.nsave = len(rg)
                nxt.append(len(segs) + 1 if k + 1 < len(rgs) else -1)
                segs.append(seg)
                saveat.extend(ts[rg.start:rg.stop].tolist())
                idx.extend(range(rg.start, rg.stop))
                self.groups.append((ti, rg))
            self.cols.append(np.asarray(idx, dtype=np.int64))
            self.starts.append(np.asarray([rg.start for rg in rgs], dtype=np.int64))
        self.segs = (_lib.Segment * len(segs))(*segs)
        self.saveat = np.ascontiguousarray(saveat, dtype=np.float64)
        self.seg_next = np.ascontiguousarray(nxt, dtype=np.int32)
        self.nseg = len(segs)
        # the same indices into the trajectories' data concatenated along time
        self.lengths = np.asarray([len(ts) for ts, _ in shapes], dtype=np.int64)
        offs = np.concatenate([[0], np.cumsum(self.lengths)[:-1]]).astype(np.int64)
        self.gcols = np.concatenate([c + o for c, o in zip(self.cols, offs)])
        self.gstarts = np.concatenate([st + o for st, o in zip(self.starts, offs)])
        # every trajectory's times, concatenated: a cached layout is reused
        # only for the same times
        self.tcat = np.concatenate([np.asarray(ts, dtype=np.float64) for ts, _ in shapes])


class _Packed:
    """Segment table and packed values (initial states, data at the saves) of
    one or many trajectories; the table is reused across calls with the same
    lengths, group sizes and times."""

    _cache = {}

    def __init__(self, trajectories):
        # trajectories: list of (data S x n, tsteps n, group_size)
        key = tuple((len(ts), int(gs)) for _, ts, gs in trajectories)
        lay = _Packed._cache.get(key)
        if lay is not None:
            tcat = np.concatenate([np.asarray(ts, dtype=np.float64) for _, ts, _ in trajectories])
            if not np.array_equal(tcat, lay.tcat):
                lay = None
        if lay is None:
            lay = _Layout([(ts, gs) for _, ts, gs in trajectories])
            _Packed._cache = {key: lay}  # keep the last layout only
        self.layout = lay
        self.segs, self.saveat, self.nseg, self.groups = lay.segs, lay.saveat, lay.nseg, lay.groups
        ds = [np.asarray(d, dtype=np.float32) for d, _, _ in trajectories]
        for d, n in zip(ds, lay.lengths):
            if d.ndim != 2 or d.shape[1] != n:
                raise ValueError(f"trajectory data of shape {d.shape} does not have {n} time points")
        # u0: nseg x S (column-major S x nseg); data at the saves: nsave_total x S,
        # both gathered as rows of the time-major view of the concatenated data
        allT = np.concatenate(ds, axis=1).T
        self.u0 = allT[lay.gstarts]
        self.data = allT[lay.gcols]


class MultipleShooter:
    """Packed forward and discrete-adjoint backward of multiple-shooting groups."""

    def __init__(self, solver, abstol=1e-6, reltol=1e-3, maxiters=100000):
        self.solver = solver
        self.abstol, self.reltol, self.maxiters = float(abstol), float(reltol), int(maxiters)

    def forward(self, packed, p, fetch=True):
        """Solves every segment; returns (saves S x nsave_total, or None when
        fetch is False and they stay on the device, retcodes, stats)."""
        s = self.solver
        if hasattr(p, "is_cuda") and p.is_cuda:
            s.set_params_device(p.detach().to(dtype=__import__("torch").float32).contiguous())
        else:
            s.set_params(p.detach().cpu().numpy() if hasattr(p, "detach") else p)
        S = s.state_dim
        out = np.empty((len(packed.saveat), S), dtype=np.float32) if fetch else None
        ret = np.zeros(packed.nseg, dtype=np.int32)
        st = _lib.Stats()
        s.bump()
        _lib.check(s.lib.gbnde_multishoot_forward(
            s.h, S, packed.nseg, packed.segs, packed.saveat.ctypes.data_as(C.POINTER(C.c_double)),
            len(packed.saveat), packed.u0.ctypes.data, self.abstol, self.reltol, self.maxiters,
            None if out is None else out.ctypes.data, ret.ctypes.data_as(C.POINTER(C.c_int)), C.byref(st)))
        return (None if out is None else out.T), ret, st  # S x nsave_total

    def saves(self, packed):
        """The saves of the last forward (S x nsave_total), copied from the device."""
        s = self.solver
        out = np.empty((len(packed.saveat), s.state_dim), dtype=np.float32)
        _lib.check(s.lib.gbnde_multishoot_saves(s.h, out.ctypes.data))
        return out.T

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

    def loss(self, packed, kind, continuity_term):
        """gbnde_multishoot_loss on the saves of the last forward; the cotangent stays on the device."""
        s = self.solver
        out = C.c_double()
        _lib.check(s.lib.gbnde_multishoot_loss(s.h, packed.data.ctypes.data, packed.layout.seg_next.ctypes.data,
                                               int(kind), float(continuity_term), C.byref(out)))
        return out.value

    def backward_fused(self):
        """dL/dp of the last gbnde_multishoot_loss (its cotangent never leaves the device)."""
        s = self.solver
        dp = np.empty(s.nparams, dtype=np.float32)
        st = _lib.Stats()
        _lib.check(s.lib.gbnde_multishoot_backward(s.h, None, None, dp.ctypes.data, C.byref(st)))
        return dp


class _Groups:
    """The group predictions (S x len(range) each), sliced from the packed saves
    on access. `us` is the S x nsave_total array, or a function returning it
    (called once, on the first access)."""

    def __init__(self, us, groups, segs):
        self._src, self._groups, self._segs = us, groups, segs
        self._arr = None

    @property
    def _us(self):
        if self._arr is None:
            self._arr = self._src() if callable(self._src) else self._src
        return self._arr

    def __len__(self):
        return len(self._groups)

    def __getitem__(self, k):
        if isinstance(k, slice):
            return [self[i] for i in range(*k.indices(len(self)))]
        seg = self._segs[k]
        return self._us[:, seg.save_off:seg.save_off + seg.nsave]

    def __iter__(self):
        return (self[k] for k in range(len(self)))


def _fused_loss(shooter, packed, p, kind, continuity_term):
    """Forward of every group, loss and continuity terms in one kernel, and
    (with a torch p) the adjoint as the loss's backward. Returns (loss, preds)."""
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    # the saves stay on the device; the predictions are copied out on first use
    _, ret, _ = shooter.forward(packed, p, fetch=False)
    shooter._nseg = packed.nseg
    solver = shooter.solver
    gen = solver.generation

    def fetch():
        if solver.generation != gen:
            # another solve ran on the context since: this call's forward again
            return shooter.forward(packed, p)[0]
        return shooter.saves(packed)
    preds = _Groups(fetch, packed.groups, packed.segs)
    if np.any(ret != 0):
        return math.inf, preds
    L = shooter.loss(packed, kind, continuity_term)
    if torch is None or not isinstance(p, torch.Tensor):
        return L, preds

    class _Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, pt):
            return torch.tensor(L, dtype=torch.float64, device=pt.device)

        @staticmethod
        def backward(ctx, g):
            if solver.generation != gen:
                # another solve ran on the context: this call's forward and
                # loss are solved again (deterministic: the same cotangent)
                shooter.forward(packed, p)
                shooter.loss(packed, kind, continuity_term)
            dp = torch.from_numpy(shooter.backward_fused()).to(g.device)
            return (g.to(torch.float32) * dp).to(p.dtype)

    return _Fn.apply(p), preds


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
                ctx.pn = pt.detach().cpu().numpy()
                us, ret, st = shooter.forward(packed, ctx.pn)
                shooter._nseg = packed.nseg
                ctx.ret = ret
                ctx.generation = shooter.solver.generation
                return torch.from_numpy(np.ascontiguousarray(us)).to(pt.device), torch.from_numpy(ret)

            @staticmethod
            def backward(ctx, g, _gret):
                if np.any(ctx.ret != 0):
                    raise RuntimeError("cannot differentiate multiple shooting with a failed group")
                if shooter.solver.generation != ctx.generation:
                    shooter.forward(packed, ctx.pn)  # another solve ran since: solve this one again
                    shooter._nseg = packed.nseg
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
    packed = _Packed(trajectories)
    shooter = MultipleShooter(solver, abstol, reltol, maxiters)
    try:
        kind = _FUSED_KIND.get(loss_function)
    except TypeError:  # an unhashable loss object
        kind = None
    if kind is not None and continuity_loss is None:
        # sum/mean of squares with the default continuity loss: the whole loss
        # on the device, no per-group host work
        return _fused_loss(shooter, packed, p, kind, continuity_term)
    if continuity_loss is None:
        continuity_loss = _default_continuity_loss
    us, ret = _predict(shooter, packed, p)
    preds_loss, preds = _loss(packed, us, trajectories, loss_function, continuity_loss, continuity_term)
    if np.any(ret != 0):
        return math.inf, preds
    return preds_loss, preds
