"""Host-side mirror of DiffEqFlux's FFJORD layer on the GB300 solver.

`FFJORD(model, tspan, input_dims, alg; basedist=None, kwargs...)` and
`(f)(x, ps, st) -> ((logpx, lambda1, lambda2), st)` as in src/ffjord.jl:51-178:
the augmented system [z; delta_logp] with right-hand side
[f(z [, t]); -trace(df/dz)] is solved from (x, 0), keeping only the end state,
and logpx = logpz(z(t1)) - delta_logp(t1) with the standard-normal base.
`st` carries the reference's flags: monte_carlo (Hutchinson trace, the
default) or the exact trace, and regularize: two more rows integrate |f|^2
and |e^T J| (src/ffjord.jl:131-132), returned as lambda1 and lambda2 (1 x B
each) and differentiable like logpx. (The reference selects its lambda1 and
lambda2 along the batch dimension of the end state, src/ffjord.jl:164-166,
which returns batch columns rather than those two rows; the reference's tests
use only logpx. This layer returns the two rows.) `basedist` is the
base density: None for the standard normal, or an object with
``logpdf(z) -> (B,)`` on z of shape (d, B) (a torch-differentiable function of
z when the layer is called with torch tensors); logpx = basedist.logpdf(z(t1))
- delta_logp(t1) (src/ffjord.jl:170-176), differentiated through the
library's dL/dz(t1). Like the reference without regularisation, the layer
returns (logpx, delta_logp, delta_logp). The Hutchinson
noise is drawn once per sample per solve (Rademacher by default, Gaussian on
request) from `st["rng"]` -- the reference draws fresh Gaussian noise on every
right-hand-side call, which makes its ODE stochastic. With torch tensors the
returned logpx is differentiable through the library's InterpolatingAdjoint.
"""
import ctypes as C

import numpy as np

from . import _lib
from .layers import Chain, Solver, Tsit5


class FFJORD:
    def __init__(self, model, tspan, input_dims, alg=None, *, basedist=None, abstol=1e-6, reltol=1e-3,
                 maxiters=100000, time_input=False, noise="rademacher", device=0):
        if not isinstance(model, Chain):
            raise TypeError("model must be a Chain of Dense layers")
        if basedist is not None and not callable(getattr(basedist, "logpdf", None)):
            raise TypeError("basedist must be None (standard normal) or have logpdf(z) -> (B,)")
        self.basedist = basedist
        if model.cube_input:
            raise ValueError("FFJORD models take no cube prefix")
        d = int(np.prod(input_dims))
        if model.dims[-1] != d or model.dims[0] != d + (1 if time_input else 0):
            raise ValueError("model must map the data dim (plus t when time_input) to the data dim")
        self.model, self.d = model, d
        self.tspan = (float(tspan[0]), float(tspan[1]))
        self.alg = alg if alg is not None else Tsit5()
        self.abstol, self.reltol, self.maxiters = float(abstol), float(reltol), int(maxiters)
        self.time_input = bool(time_input)
        self.noise = noise
        self.device = device
        self._solver = None

    # Lux.initialstates (src/ffjord.jl:61-66)
    def setup(self, rng):
        return self.model.init_params(rng), {"regularize": False, "monte_carlo": True,
                                             "rng": np.random.default_rng(int(rng.integers(1 << 31)))}

    @property
    def solver(self):
        if self._solver is None:
            self._solver = Solver(self.model, self.alg.precision, self.device, time_input=self.time_input)
        return self._solver

    def desc(self):
        return Solver.solve_desc(self.tspan[0], self.tspan[1], [self.tspan[1]], self.abstol, self.reltol,
                                 0, 0.0, 0.0, self.maxiters)

    def draw_noise(self, rng, B):
        if self.noise == "gaussian":
            return rng.standard_normal((B, self.d)).astype(np.float32)
        return rng.choice(np.array([-1.0, 1.0], np.float32), size=(B, self.d))

    # numpy core --------------------------------------------------------------------
    def forward_np(self, x, p, noise):
        """x: d x B. noise: B x d (row-major per sample) or None (exact trace)."""
        s = self.solver
        s.set_params(p)
        x = np.ascontiguousarray(np.asarray(x, np.float32).T)  # B x d = column-major d x B
        B = x.shape[0]
        logpx = np.empty(B, np.float32)
        zT = np.empty((B, self.d), np.float32)
        st = _lib.Stats()
        nz = None if noise is None else np.ascontiguousarray(noise, np.float32)
        s.bump()
        _lib.check(s.lib.gbnde_ffjord_forward(s.h, C.byref(self.desc()), self.d, B, x.ctypes.data,
                                              None if nz is None else nz.ctypes.data, logpx.ctypes.data,
                                              zT.ctypes.data, C.byref(st)))
        self._keep = nz
        return logpx, zT.T, st

    def forward_reg_np(self, x, p, noise, exact):
        """regularize = true: returns (logpx, z(t1), |f|^2 integral, |e^T J|
        integral, stats); noise (B x d) is the e of |e^T J| and, unless exact,
        the Hutchinson direction."""
        s = self.solver
        s.set_params(p)
        x = np.ascontiguousarray(np.asarray(x, np.float32).T)
        B = x.shape[0]
        logpx = np.empty(B, np.float32)
        zT = np.empty((B, self.d), np.float32)
        rf = np.empty(B, np.float32)
        rj = np.empty(B, np.float32)
        st = _lib.Stats()
        nz = np.ascontiguousarray(noise, np.float32)
        s.bump()
        _lib.check(s.lib.gbnde_ffjord_forward_reg(s.h, C.byref(self.desc()), self.d, B, x.ctypes.data,
                                                  nz.ctypes.data, 1 if exact else 0, logpx.ctypes.data,
                                                  zT.ctypes.data, rf.ctypes.data, rj.ctypes.data, C.byref(st)))
        self._keep = nz
        return logpx, zT.T, rf, rj, st

    def backward_reg_np(self, dlogpx, dzT=None, drf=None, drj=None):
        s = self.solver
        g = np.ascontiguousarray(dlogpx, np.float32)
        B = g.size
        opt = lambda a: None if a is None else np.ascontiguousarray(np.asarray(a, np.float32))  # noqa: E731
        gz = None if dzT is None else np.ascontiguousarray(np.asarray(dzT, np.float32).T)
        gf, gj = opt(drf), opt(drj)
        dx = np.empty((B, self.d), np.float32)
        dp = np.empty(s.nparams, np.float32)
        st = _lib.Stats()
        ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        _lib.check(s.lib.gbnde_ffjord_backward_reg(s.h, g.ctypes.data, ptr(gz), ptr(gf), ptr(gj),
                                                   dx.ctypes.data, dp.ctypes.data, C.byref(st)))
        return dx.T, dp, st

    def logpz_std(self, z):
        """log density of the standard-normal base at z (d x B): the library's logpx uses it."""
        return -0.5 * (z ** 2).sum(0) - 0.5 * self.d * np.log(2.0 * np.pi)

    def backward_np(self, dlogpx, dzT=None):
        s = self.solver
        g = np.ascontiguousarray(dlogpx, np.float32)
        B = g.size
        gz = None if dzT is None else np.ascontiguousarray(np.asarray(dzT, np.float32).T)
        dx = np.empty((B, self.d), np.float32)
        dp = np.empty(s.nparams, np.float32)
        st = _lib.Stats()
        _lib.check(s.lib.gbnde_ffjord_backward(s.h, g.ctypes.data, None if gz is None else gz.ctypes.data,
                                               dx.ctypes.data, dp.ctypes.data, C.byref(st)))
        return dx.T, dp, st

    def __call__(self, x, ps, st):
        if st.get("regularize", False):
            return self._call_reg(x, ps, st)
        mc = st.get("monte_carlo", True)
        rng = st.get("rng") or np.random.default_rng(0)
        B = np.asarray(x.shape)[-1]
        noise = self.draw_noise(rng, int(B)) if mc else None
        try:
            import torch
            is_torch = isinstance(x, torch.Tensor) or isinstance(ps, torch.Tensor)
        except ImportError:  # pragma: no cover
            is_torch = False
        if not is_torch:
            logpx, zT, _ = self.forward_np(x, ps, noise)
            delta = self.logpz_std(zT.astype(np.float64)) - logpx
            if self.basedist is not None:
                logpx = np.asarray(self.basedist.logpdf(zT)) - delta
            out = logpx.reshape(1, -1)
            dl = delta.reshape(1, -1)
            return (out, dl, dl), st
        import torch
        layer = self

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, xt, pt):
                ctx.inputs = (xt.detach().cpu().numpy(), pt.detach().cpu().numpy())
                lp, zT, _ = layer.forward_np(ctx.inputs[0], ctx.inputs[1], noise)
                ctx.generation = layer.solver.generation
                return torch.from_numpy(lp).to(pt.device), torch.from_numpy(np.ascontiguousarray(zT)).to(pt.device)

            @staticmethod
            def backward(ctx, g, gz):
                if layer.solver.generation != ctx.generation:
                    # another solve ran on the context since this forward: the
                    # adjoint needs this call's own solve, so it is run again
                    layer.forward_np(ctx.inputs[0], ctx.inputs[1], noise)
                dx, dp, _ = layer.backward_np(g.detach().cpu().numpy(),
                                              None if gz is None else gz.detach().cpu().numpy())
                return torch.from_numpy(np.ascontiguousarray(dx)).to(g.device), torch.from_numpy(dp).to(g.device)

        xt = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x, np.float32))
        pt = ps if isinstance(ps, torch.Tensor) else torch.as_tensor(np.asarray(ps, np.float32))
        lp_std, zT = _Fn.apply(xt, pt)
        delta = (-0.5 * (zT.double() ** 2).sum(0) - 0.5 * self.d * np.log(2.0 * np.pi)) - lp_std.double()
        if self.basedist is not None:
            lp = (self.basedist.logpdf(zT).double() - delta).to(lp_std.dtype)
        else:
            lp = lp_std
        dl = delta.to(lp_std.dtype).reshape(1, -1)
        return (lp.reshape(1, -1), dl, dl), st


    def _call_reg(self, x, ps, st):
        """regularize = true: (logpx, lambda1, lambda2) with lambda1 = the
        integral of |f|^2 and lambda2 = that of |e^T J| (1 x B each)."""
        exact = not st.get("monte_carlo", True)
        rng = st.get("rng") or np.random.default_rng(0)
        B = int(np.asarray(x.shape)[-1])
        noise = self.draw_noise(rng, B)
        try:
            import torch
            is_torch = isinstance(x, torch.Tensor) or isinstance(ps, torch.Tensor)
        except ImportError:  # pragma: no cover
            is_torch = False
        if not is_torch:
            logpx, zT, rf, rj, _ = self.forward_reg_np(x, ps, noise, exact)
            if self.basedist is not None:
                delta = self.logpz_std(zT.astype(np.float64)) - logpx
                logpx = np.asarray(self.basedist.logpdf(zT)) - delta
            return (logpx.reshape(1, -1), rf.reshape(1, -1), rj.reshape(1, -1)), st
        import torch
        layer = self

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, xt, pt):
                ctx.inputs = (xt.detach().cpu().numpy(), pt.detach().cpu().numpy())
                lp, zT, rf, rj, _ = layer.forward_reg_np(ctx.inputs[0], ctx.inputs[1], noise, exact)
                ctx.generation = layer.solver.generation
                dev = pt.device
                return (torch.from_numpy(lp).to(dev), torch.from_numpy(np.ascontiguousarray(zT)).to(dev),
                        torch.from_numpy(rf).to(dev), torch.from_numpy(rj).to(dev))

            @staticmethod
            def backward(ctx, g, gz, gf, gj):
                if layer.solver.generation != ctx.generation:
                    layer.forward_reg_np(ctx.inputs[0], ctx.inputs[1], noise, exact)
                host = lambda a: None if a is None else a.detach().cpu().numpy()  # noqa: E731
                dx, dp, _ = layer.backward_reg_np(host(g), host(gz), host(gf), host(gj))
                return torch.from_numpy(np.ascontiguousarray(dx)).to(g.device), torch.from_numpy(dp).to(g.device)

        xt = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x, np.float32))
        pt = ps if isinstance(ps, torch.Tensor) else torch.as_tensor(np.asarray(ps, np.float32))
        lp_std, zT, rf, rj = _Fn.apply(xt, pt)
        if self.basedist is not None:
            delta = (-0.5 * (zT.double() ** 2).sum(0) - 0.5 * self.d * np.log(2.0 * np.pi)) - lp_std.double()
            lp = (self.basedist.logpdf(zT).double() - delta).to(lp_std.dtype)
        else:
            lp = lp_std
        return (lp.reshape(1, -1), rf.reshape(1, -1), rj.reshape(1, -1)), st


class FFJORDDistribution:
    """``FFJORDDistribution(model, ps, st)`` (src/ffjord.jl:217-246): `rand` solves
    the flow backwards in time from base samples (``reverse(tspan)``, :183-214)
    and returns z; `logpdf` is the forward logpx."""

    def __init__(self, model, ps, st):
        self.model, self.ps, self.st = model, ps, st
        self._rev = FFJORD(model.model, (model.tspan[1], model.tspan[0]), (model.d,), model.alg,
                           abstol=model.abstol, reltol=model.reltol, maxiters=model.maxiters,
                           time_input=model.time_input, noise=model.noise, device=model.device)

    def __len__(self):
        return self.model.d

    def logpdf(self, x):
        x = np.asarray(x, np.float32)
        x2 = x.reshape(-1, 1) if x.ndim == 1 else x
        (lp, _, _), _ = self.model(x2, self.ps, self.st)
        out = np.asarray(lp).reshape(-1)
        return out[0] if x.ndim == 1 else out

    def pdf(self, x):
        return np.exp(self.logpdf(x))

    def rand(self, n, rng=None):
        rng = rng or self.st.get("rng") or np.random.default_rng(0)
        x = rng.standard_normal((self.model.d, n)).astype(np.float32)
        mc = self.st.get("monte_carlo", True)
        noise = self._rev.draw_noise(rng, n)
        if self.st.get("regularize", False):
            # the regulariser rows ride along (and enter the step-size control)
            # as in the reference's reversed solve (src/ffjord.jl:192-213)
            _, zT, _, _, st = self._rev.forward_reg_np(x, self.ps, noise, not mc)
        else:
            _, zT, st = self._rev.forward_np(x, self.ps, noise if mc else None)
        _lib.check(0 if st.retcode == 0 else _lib.ERR_INVALID)
        return zT
