"""Host-side mirror of the DiffEqFlux NeuralODE layer on the GB300 solver.

Python counterpart of the Julia glue: the layer keeps the reference's
constructor and call, ``NeuralODE(model, tspan, alg; saveat, abstol, reltol,
sensealg, ...)`` and ``node(x, p, st) -> (sol, st)`` (src/neural_de.jl:35-61),
and routes the solve to libgbnde.so. The model is a ``Chain`` of an optional
cube ``WrappedFunction`` and ``Dense`` layers, as in
docs/src/examples/neural_ode.md:32 and test/BasicNeuralDE/neural_de_tests.jl:17.
Anything else raises: there is no CPU fallback.

Differentiation: ``solve_saveat`` is a ``torch.autograd.Function`` whose
backward runs the library's adjoint kernel (the role SciMLSensitivity's
``rrule`` on ``solve`` plays for Zygote in the reference).
"""
import ctypes as C
import math

import numpy as np

from . import _lib

# ---------------------------------------------------------------------------
# model description (Lux-like)
# ---------------------------------------------------------------------------


class Dense:
    """``Dense(in, out, act)``: y = act.(W*x .+ b), W is out x in."""

    def __init__(self, in_dims, out_dims, activation="identity"):
        if isinstance(in_dims, tuple):  # Dense(in => out) written as a pair
            in_dims, out_dims = in_dims
        self.in_dims = int(in_dims)
        self.out_dims = int(out_dims)
        if callable(activation):
            activation = getattr(activation, "__name__", str(activation))
        if activation not in _lib.ACT:
            raise ValueError(f"unsupported activation {activation!r}; use identity/tanh/softplus")
        self.activation = activation


class WrappedFunction:
    """``WrappedFunction(x -> x.^3)``: only the elementwise cube is supported."""

    def __init__(self, kind="cube"):
        if kind != "cube":
            raise ValueError("only the x -> x.^3 WrappedFunction is supported")
        self.kind = kind


def cube():
    return WrappedFunction("cube")


class Chain:
    def __init__(self, *layers):
        self.layers = list(layers)
        dense = [l for l in self.layers if isinstance(l, Dense)]
        if not dense:
            raise ValueError("Chain needs at least one Dense layer")
        for i, l in enumerate(self.layers):
            if isinstance(l, WrappedFunction) and i != 0:
                raise ValueError("the cube WrappedFunction must come first in the Chain")
            if not isinstance(l, (Dense, WrappedFunction)):
                raise TypeError(f"unsupported layer {type(l).__name__}")
        for a, b in zip(dense, dense[1:]):
            if a.out_dims != b.in_dims:
                raise ValueError("Dense dimensions do not chain")
        self.dense = dense
        self.cube_input = isinstance(self.layers[0], WrappedFunction)

    @property
    def dims(self):
        return [self.dense[0].in_dims] + [d.out_dims for d in self.dense]

    @property
    def acts(self):
        return [d.activation for d in self.dense]

    def nparams(self):
        return sum(d.in_dims * d.out_dims + d.out_dims for d in self.dense)

    def desc(self, time_input=False):
        d = _lib.MlpDesc()
        d.nlayers = len(self.dense)
        for i, v in enumerate(self.dims):
            d.dims[i] = v
        for i, a in enumerate(self.acts):
            d.act[i] = _lib.ACT[a]
        d.cube_input = int(self.cube_input)
        d.time_input = int(time_input)
        return d

    def init_params(self, rng, dtype=np.float32):
        """Glorot-uniform weights, zero biases, flat ComponentArray order."""
        parts = []
        for d in self.dense:
            lim = math.sqrt(6.0 / (d.in_dims + d.out_dims))
            W = rng.uniform(-lim, lim, size=(d.out_dims, d.in_dims))
            parts.append(W.T.reshape(-1))       # column-major out x in
            parts.append(np.zeros(d.out_dims))
        return np.concatenate(parts).astype(dtype)


# ---------------------------------------------------------------------------
# algorithm / sensealg markers (re-exports of the reference, src/DiffEqFlux.jl:53-56)
# ---------------------------------------------------------------------------


class ZygoteVJP:
    """VJP backend marker; the VJP is the library's fused transpose GEMMs."""


class InterpolatingAdjoint:
    code = _lib.SENSE["interpolating"]

    def __init__(self, autojacvec=None, checkpointing=False):
        self.autojacvec = autojacvec
        self.checkpointing = checkpointing


class BacksolveAdjoint:
    code = _lib.SENSE["backsolve"]

    def __init__(self, autojacvec=None, checkpointing=True):
        self.autojacvec = autojacvec
        self.checkpointing = checkpointing


class GaussAdjoint:
    """Quadrature adjoint: the backward solve carries lam only, and dL/dp is
    integrated by 4-point Gauss-Legendre over every accepted adjoint step
    (lam from the step's interpolant, u from the forward's dense output).
    Runs in the FP32 adjoint kernel in both precision forms."""
    code = _lib.SENSE["gauss"]

    def __init__(self, autojacvec=None, checkpointing=False):
        self.autojacvec = autojacvec
        self.checkpointing = checkpointing


class QuadratureAdjoint(GaussAdjoint):
    """QuadratureAdjoint(abstol, reltol): the reference integrates the
    parameter quadrature with adaptive Gauss-Kronrod over each save interval
    on a stored lam interpolant; here the same integral is taken with the
    per-step Gauss-Legendre rule of GaussAdjoint (exact to the interpolant's
    order), so abstol/reltol of the quadrature are accepted and unused."""

    def __init__(self, autojacvec=None, abstol=1e-6, reltol=1e-3):
        super().__init__(autojacvec)
        self.abstol, self.reltol = abstol, reltol


class Tsit5:
    """Tsit5 marker routing the solve to the GB300 kernels.

    precision="fp32": plain FP32 everywhere (the drop-in form);
    precision="bf16": tensor-core BF16 GEMMs with FP32 state and FP64 control.
    """

    def __init__(self, precision="fp32"):
        if precision not in _lib.PREC:
            raise ValueError("precision must be 'fp32' or 'bf16'")
        self.precision = precision


GB300Tsit5 = Tsit5


# ---------------------------------------------------------------------------
# solver context cache
# ---------------------------------------------------------------------------


class Solver:
    """One library context: a model, a precision and a device."""

    def __init__(self, model, precision="fp32", device=0, time_input=False):
        self.lib = _lib.load()
        self.model = model
        self.desc = model.desc(time_input)
        h = C.c_void_p()
        _lib.check(self.lib.gbnde_create(C.byref(h), C.byref(self.desc), _lib.PREC[precision], int(device)))
        self.h = h
        self.nparams = int(self.lib.gbnde_nparams(h))
        self.state_dim = model.dims[-1]
        # Count of solves run on this context. The library's backward
        # differentiates the context's LAST forward solve; an autograd node
        # records the count of its own forward and re-solves when another
        # forward (or a training step) has run since.
        self.generation = 0

    def bump(self):
        """Marks that a call replaced the context's last forward solve."""
        self.generation += 1
        return self.generation

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbnde_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- numpy (host pointer) path -------------------------------------------
    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _lib.check(self.lib.gbnde_set_params(self.h, p.ctypes.data, p.size))

    @staticmethod
    def solve_desc(t0, t1, saveat, abstol, reltol, sensealg=0, dt0=0.0, dtmin=0.0, maxiters=100000, flags=0):
        sv = np.ascontiguousarray(saveat, dtype=np.float64)
        d = _lib.SolveDesc()
        d.t0, d.t1 = float(t0), float(t1)
        d.abstol, d.reltol = float(abstol), float(reltol)
        d.dt0, d.dtmin = float(dt0), float(dtmin)
        d.maxiters = int(maxiters)
        d.saveat = sv.ctypes.data_as(C.POINTER(C.c_double))
        d.nsave = sv.size
        d.sensealg = int(sensealg)
        d.flags = int(flags)
        d._keep = sv
        return d

    def forward(self, u0, desc):
        """u0: (S, B) array. Returns (usave (S, B, nsave), stats)."""
        self.bump()
        u0 = np.asarray(u0, dtype=np.float32)
        S, B = u0.shape
        buf = np.ascontiguousarray(u0.T)            # column-major S x B
        out = np.empty((desc.nsave, B, S), dtype=np.float32)
        st = _lib.Stats()
        _lib.check(self.lib.gbnde_forward(self.h, C.byref(desc), S, B, buf.ctypes.data,
                                          out.ctypes.data, C.byref(st)))
        return np.transpose(out, (2, 1, 0)), st

    def backward(self, dL_dusave):
        """dL_dusave: (S, B, nsave). Returns (dL/du0 (S, B), dL/dp, stats)."""
        g = np.asarray(dL_dusave, dtype=np.float32)
        S, B, ns = g.shape
        buf = np.ascontiguousarray(np.transpose(g, (2, 1, 0)))
        du0 = np.empty((B, S), dtype=np.float32)
        dp = np.empty(self.nparams, dtype=np.float32)
        st = _lib.Stats()
        _lib.check(self.lib.gbnde_backward(self.h, buf.ctypes.data, du0.ctypes.data,
                                           dp.ctypes.data, C.byref(st)))
        return du0.T, dp, st

    def forward_steps(self, cap=1 << 20):
        t = np.zeros(cap)
        h = np.zeros(cap)
        n = self.lib.gbnde_forward_steps(self.h, t.ctypes.data_as(C.POINTER(C.c_double)),
                                         h.ctypes.data_as(C.POINTER(C.c_double)), cap)
        n = min(n, cap)
        return list(zip(t[:n].tolist(), h[:n].tolist()))

    def forward_trace(self, cap=1 << 20):
        """Attempted steps of the last forward: list of (t, h, EEst, accepted)."""
        buf = np.zeros(4 * cap)
        n = self.lib.gbnde_forward_trace(self.h, buf.ctypes.data_as(C.POINTER(C.c_double)), cap)
        n = min(n, cap)
        return [(buf[4 * i], buf[4 * i + 1], buf[4 * i + 2], bool(buf[4 * i + 3])) for i in range(n)]

    # -- device (torch CUDA tensor) path --------------------------------------
    def set_params_device(self, p):
        _lib.check(self.lib.gbnde_set_params_device(self.h, p.data_ptr(), p.numel()))

    def forward_device(self, u0_cm, usave_cm, desc, S, B):
        self.bump()
        st = _lib.Stats()
        _lib.check(self.lib.gbnde_forward_device(self.h, C.byref(desc), S, B, u0_cm.data_ptr(),
                                                 usave_cm.data_ptr(), C.byref(st)))
        return st

    def backward_device(self, g_cm, du0_cm, dp):
        st = _lib.Stats()
        _lib.check(self.lib.gbnde_backward_device(self.h, g_cm.data_ptr(), du0_cm.data_ptr(),
                                                  dp.data_ptr(), C.byref(st)))
        return st

    def loss_device(self, usave_cm, target_cm, kind, dl_cm):
        out = C.c_double()
        _lib.check(self.lib.gbnde_loss_device(self.h, usave_cm.data_ptr(), target_cm.data_ptr(),
                                              int(kind), dl_cm.data_ptr(), C.byref(out)))
        return out.value

    def train_step(self, u0_cm, target_cm, desc, S, B, p, m, v, step, lr=1e-3, beta1=0.9, beta2=0.999,
                   eps=1e-8, kind=1):
        """One Adam iteration on device tensors (gbnde_train_step): p, m, v are
        updated in place; returns (loss, stats)."""
        self.bump()
        opt = _lib.Adam(float(lr), float(beta1), float(beta2), float(eps))
        out = C.c_double()
        st = _lib.Stats()
        _lib.check(self.lib.gbnde_train_step(self.h, C.byref(desc), S, B, u0_cm.data_ptr(),
                                             target_cm.data_ptr(), int(kind), C.byref(opt), int(step),
                                             p.data_ptr(), m.data_ptr(), v.data_ptr(), C.byref(out),
                                             C.byref(st)))
        return out.value, st

    def graph_train_step(self, u0_cm, target_cm, desc, S, B, p, m, v, step, lr=1e-3, beta1=0.9,
                         beta2=0.999, eps=1e-8, kind=1):
        """gbnde_graph_train_step: the same iteration replayed as one CUDA graph
        after the first call; returns (loss, stats, ran_as_graph)."""
        self.bump()
        opt = _lib.Adam(float(lr), float(beta1), float(beta2), float(eps))
        out = C.c_double()
        st = _lib.Stats()
        g = C.c_int()
        _lib.check(self.lib.gbnde_graph_train_step(self.h, C.byref(desc), S, B, u0_cm.data_ptr(),
                                                   target_cm.data_ptr(), int(kind), C.byref(opt), int(step),
                                                   p.data_ptr(), m.data_ptr(), v.data_ptr(), C.byref(out),
                                                   C.byref(st), C.byref(g)))
        return out.value, st, bool(g.value)

    def autotune(self, u0_cm, desc, S, B):
        """gbnde_autotune: times the FP32 kernels at each rows-per-tile choice on
        this shape and keeps the fastest; returns (forward, adjoint) tile rows."""
        self.bump()
        t = (C.c_int * 2)()
        _lib.check(self.lib.gbnde_autotune(self.h, C.byref(desc), S, B, u0_cm.data_ptr(), t))
        return int(t[0]), int(t[1])


# ---------------------------------------------------------------------------
# solution type
# ---------------------------------------------------------------------------


class ODESolution:
    """Saved states and times of one solve (``sol.u``, ``sol.t``, ``Array(sol)``)."""

    def __init__(self, t, arr, retcode, stats):
        self.t = list(t)
        self._arr = arr            # (S, B, nsave)  (numpy or torch)
        self.retcode = _lib.RETCODE_NAMES.get(retcode, str(retcode))
        self.stats = stats

    @property
    def u(self):
        return [self._arr[..., i] for i in range(self._arr.shape[-1])]

    def array(self):
        return self._arr

    def __array__(self, dtype=None):
        a = np.asarray(self._arr.detach().cpu() if hasattr(self._arr, "detach") else self._arr)
        return a.astype(dtype) if dtype is not None else a

    def __len__(self):
        return len(self.t)

    def __getitem__(self, i):
        return self._arr[..., i]

    def successful(self):
        return self.retcode == "Success"


def Array(sol):  # noqa: N802  (mirrors Julia's Array(sol))
    return sol.array()


# ---------------------------------------------------------------------------
# the layer
# ---------------------------------------------------------------------------


def _saveat_points(tspan, saveat, save_start, save_end):
    t0, t1 = float(tspan[0]), float(tspan[1])
    if saveat is None or (np.ndim(saveat) > 0 and len(saveat) == 0):
        pts = []
        if save_start:
            pts.append(t0)
        if save_end or not pts:
            pts.append(t1)
        return pts
    if np.ndim(saveat) == 0:
        dt = float(saveat)
        n = int(math.floor((t1 - t0) / dt + 1e-9))
        pts = [t0 + i * dt for i in range(n + 1)]
        if save_end and abs(pts[-1] - t1) > 1e-12 * max(1.0, abs(t1)):
            pts.append(t1)
    else:
        pts = [float(s) for s in saveat]
    if save_start is False and pts and pts[0] == t0:
        pts = pts[1:]
    return pts


class NeuralODE:
    """``NeuralODE(model, tspan, alg; saveat, abstol, reltol, sensealg, ...)``.

    Mirrors src/neural_de.jl:35-61. Call ``node(x, p, st)`` with ``x`` of
    shape (S,) or (S, B) (numpy or torch) and the flat parameter vector ``p``;
    returns ``(ODESolution, st)``. With torch inputs the saved states are a
    differentiable tensor whose backward runs the adjoint kernel.
    """

    def __init__(self, model, tspan, alg=None, *, saveat=None, abstol=1e-6, reltol=1e-3,
                 sensealg=None, dt=0.0, dtmin=0.0, maxiters=100000, save_everystep=None,
                 save_start=None, save_end=True, device=0, float32_time=None):
        if not isinstance(model, Chain):
            raise TypeError("model must be a Chain of Dense layers (optionally starting with cube())")
        if alg is None:
            alg = Tsit5()
        if not isinstance(alg, Tsit5):
            raise TypeError("alg must be Tsit5()/GB300Tsit5(); other solvers are not on the GB300 path")
        if sensealg is None:
            sensealg = InterpolatingAdjoint(autojacvec=ZygoteVJP())
        if not isinstance(sensealg, (InterpolatingAdjoint, BacksolveAdjoint, GaussAdjoint)):
            raise TypeError("sensealg must be InterpolatingAdjoint(), BacksolveAdjoint(), GaussAdjoint() or "
                            "QuadratureAdjoint()")
        # the reference saves every step when no saveat is given
        # (save_everystep defaults to true then); with saveat it saves only there
        self.save_everystep = (saveat is None) if save_everystep is None else bool(save_everystep)
        self.model = model
        # A Float32 tspan makes the reference's integrator keep t and dt in
        # Float32; the FP32 form follows (GBNDE_FLAG_FP32_TIME), the BF16 form
        # keeps FP64 time by design.
        if float32_time is None:
            float32_time = (alg.precision == "fp32" and all(isinstance(x, np.float32) for x in tspan))
        if float32_time and alg.precision != "fp32":
            raise ValueError("float32_time is a mode of the FP32 form")
        self.float32_time = bool(float32_time)
        self.tspan = (float(tspan[0]), float(tspan[1]))
        self.alg = alg
        self.sensealg = sensealg
        self.abstol, self.reltol = float(abstol), float(reltol)
        self.dt, self.dtmin, self.maxiters = float(dt), float(dtmin), int(maxiters)
        if save_start is None:
            save_start = saveat is not None or self.save_everystep
        self.save_start, self.save_end = bool(save_start), bool(save_end)
        self.saveat = _saveat_points(self.tspan, saveat, save_start, save_end)
        if self.float32_time:
            self.saveat = [float(np.float32(s)) for s in self.saveat]
        self.device = device
        self._solver = None

    # Lux.setup(rng, node)
    def setup(self, rng):
        return self.model.init_params(rng), {}

    @property
    def solver(self):
        if self._solver is None:
            self._solver = Solver(self.model, self.alg.precision, self.device)
        return self._solver

    def desc(self):
        return Solver.solve_desc(self.tspan[0], self.tspan[1], self.saveat, self.abstol, self.reltol,
                                 self.sensealg.code, self.dt, self.dtmin, self.maxiters,
                                 flags=_lib.FLAG_FP32_TIME if self.float32_time else 0)

    def _everystep_points(self, x2, p, is_torch):
        """save_everystep: the accepted step times of this solve. The save points
        do not influence the step sizes (only the end of the span clips a
        step), so a first solve gives the steps, and the solve that saves at
        exactly those times (each a step end: the state itself, no
        interpolation) takes the same steps."""
        s = self.solver
        d = Solver.solve_desc(self.tspan[0], self.tspan[1], [self.tspan[1]], self.abstol, self.reltol,
                              self.sensealg.code, self.dt, self.dtmin, self.maxiters,
                              flags=_lib.FLAG_FP32_TIME if self.float32_time else 0)
        if is_torch:
            import torch
            pc = p.detach().to(torch.float32).contiguous()
            if x2.is_cuda:
                S, B = x2.shape
                u0_cm = x2.detach().to(torch.float32).t().contiguous()
                out = torch.empty((1, B, S), dtype=torch.float32, device=x2.device)
                torch.cuda.current_stream(x2.device).synchronize()
                s.set_params_device(pc.to(x2.device))
                s.forward_device(u0_cm, out, d, S, B)
            else:
                s.set_params(pc.cpu().numpy())
                s.forward(x2.detach().cpu().numpy(), d)
        else:
            s.set_params(p)
            s.forward(x2, d)
        steps = s.forward_steps()
        # each step's end is the next step's start time (as the integrator
        # stored it, Float32 time included); the last ends at t1
        ends = [steps[i + 1][0] for i in range(len(steps) - 1)] + ([self.tspan[1]] if steps else [])
        pts = ([self.tspan[0]] if self.save_start else []) + ends
        if not self.save_end and pts and pts[-1] == self.tspan[1]:
            pts = pts[:-1]
        return pts or [self.tspan[1]]

    def __call__(self, x, p, st=None):
        try:
            import torch
            is_torch = isinstance(x, torch.Tensor)
        except ImportError:  # pragma: no cover
            is_torch = False
        if self.save_everystep:
            x2 = x if (not is_torch or x.dim() == 2) else x.reshape(-1, 1)
            if not is_torch:
                x2 = np.asarray(x, dtype=np.float32)
                x2 = x2[:, None] if x2.ndim == 1 else x2
            self.saveat = self._everystep_points(x2, p, is_torch)
        if is_torch:
            from ._torch import solve_saveat
            x2 = x if x.dim() == 2 else x.reshape(-1, 1)
            arr, stats = solve_saveat(self, x2, p)
            if x.dim() == 1:
                arr = arr[:, 0, :]
        else:
            x2 = np.asarray(x, dtype=np.float32)
            one = x2.ndim == 1
            if one:
                x2 = x2[:, None]
            self.solver.set_params(p)
            arr, stats = self.solver.forward(x2, self.desc())
            if one:
                arr = arr[:, 0, :]
        return ODESolution(self.saveat, arr, stats.retcode, stats.as_dict()), st


class AugmentedNDELayer:
    """``AugmentedNDELayer(node, adim)`` (src/neural_de.jl:356-386): the state is
    padded with `adim` zero rows before the wrapped NeuralODE solves it."""

    def __init__(self, node, adim):
        self.node = node
        self.adim = int(adim)

    def setup(self, rng):
        return self.node.setup(rng)

    def augment(self, x):
        try:
            import torch
            if isinstance(x, torch.Tensor):
                z = x.new_zeros((self.adim,) + tuple(x.shape[1:]))
                return torch.cat([x, z], dim=0)
        except ImportError:  # pragma: no cover
            pass
        x = np.asarray(x, dtype=np.float32)
        return np.concatenate([x, np.zeros((self.adim,) + x.shape[1:], np.float32)], axis=0)

    def __call__(self, x, p, st=None):
        return self.node(self.augment(x), p, st)


class DimMover:
    """``DimMover(from_dim, to_dim)`` (src/neural_de.jl:397-412): moves an array
    axis (1-based, negative counts from the end), e.g. the time axis of a solution."""

    def __init__(self, from_dim=-2, to_dim=-1):
        self.from_dim, self.to_dim = from_dim, to_dim

    def __call__(self, x, p=None, st=None):
        nd = np.ndim(x)
        f = self.from_dim - 1 if self.from_dim > 0 else nd + self.from_dim
        t = self.to_dim - 1 if self.to_dim > 0 else nd + self.to_dim
        try:
            import torch
            if isinstance(x, torch.Tensor):
                return torch.movedim(x, f, t), st
        except ImportError:  # pragma: no cover
            pass
        return np.moveaxis(np.asarray(x), f, t), st
