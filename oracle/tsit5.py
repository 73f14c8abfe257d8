"""FP64 adaptive Tsit5 integrator, forward solve with saveat, and the two adjoints.

TEST INFRASTRUCTURE ONLY. This is the CPU oracle that the CUDA kernels are
checked against; the product never imports it.

What it restates
----------------
* ``NeuralODE`` forward: ``solve(ODEProblem{false}(dudt, x, tspan, p), Tsit5();
  saveat, abstol, reltol)`` (src/neural_de.jl:47-61). One adaptive integrator
  advances the whole ``S x B`` state: one step size and one RMS error norm over
  all ``S*B`` entries.
* Integrator arithmetic (OrdinaryDiffEq, not vendored; published methods):
  Tsit5 stages and embedded error (Tsitouras 2011), scaled residual
  ``utilde / (abstol + max(|uprev|, |u|) * reltol)`` with the RMS norm, the PI
  step-size controller (Hairer-Wanner II.4 / Gustafsson), the initial step of
  Hairer-Norsett-Wanner I.II.4 as the integrator implements it, the free
  interpolant for ``saveat``, and clipping of the step to the end of the span.
* Gradient with ``sensealg = InterpolatingAdjoint()`` (the default set at
  src/neural_de.jl:57) and ``BacksolveAdjoint()`` (selected at
  test/BasicNeuralDE/neural_de_tests.jl:36), from SciMLSensitivity (not
  vendored): the continuous adjoint ``dlam/dt = -J^T lam``,
  ``dmu/dt = -(df/dp)^T lam`` integrated from the last save point to ``t0``
  with the same Tsit5 tableau and tolerances, jumps ``lam += dL/du(t_i)`` at
  the save points (which are stops of the backward solve), ``u(t)`` from the
  forward dense output (Interpolating) or co-integrated backwards and reset to
  the saved forward value at each save point (Backsolve, checkpointing on).

Choices that the reference's sources here cannot settle (recorded in the
design notes as assumptions; parity with the Julia solve is unpinned):
the controller constants in ``tableau.py``; the backward error norm covers the
adjoint state (``lam``, plus ``u`` for Backsolve) but not the parameter
quadrature ``mu``; the backward solve starts at the last save point with
``lam = dL/du(t_last)`` as its initial value.
"""
import bisect
import math

import numpy as np

try:
    from . import tableau as T
except ImportError:  # pragma: no cover
    import tableau as T  # type: ignore

RET_SUCCESS = 0
RET_MAXITERS = 1
RET_DTMIN = 2
RET_UNSTABLE = 3


def _rms_sum(arrs, masks):
    s = 0.0
    n = 0
    for a, m in zip(arrs, masks):
        if m:
            s += float(np.sum(np.square(a)))
            n += a.size
    return s, n


class Tsit5:
    """Adaptive Tsit5 on a tuple of arrays ``y = (y_0, ..., y_m)``.

    ``F(y, t) -> tuple of arrays`` is the right-hand side. ``norm_mask[c]``
    says whether component ``c`` enters the error norm. ``tstops`` are times
    the integrator must hit exactly (the end of the span is always one), and
    ``on_stop(t, y) -> y or None`` is applied at each of them (a discrete
    callback); returning a new ``y`` re-evaluates the FSAL stage.
    ``steps`` replays a fixed list of ``(t_n, h_n)`` instead of adapting.
    ``time_f32`` keeps t, the step size, the error estimate and qold as
    Float32 values (rounded after each update), as the reference's integrator
    does when the time span is Float32 (src/neural_de.jl:52 builds the problem
    from the user's tspan); the state arithmetic stays FP64.
    """

    def __init__(self, F, y0, t0, t1, abstol, reltol, norm_mask=None, dt0=0.0,
                 dtmax=None, dtmin=0.0, maxiters=100000, tstops=(), on_stop=None,
                 steps=None, record=False, on_accept=None, time_f32=False):
        self.F = F
        self._r = (lambda x: float(np.float32(x))) if time_f32 else (lambda x: x)
        self.y = tuple(np.array(c, dtype=np.float64) for c in y0)
        self.t = float(t0)
        self.t0 = float(t0)
        self.t1 = float(t1)
        self.tdir = 1.0 if t1 >= t0 else -1.0
        self.abstol = float(abstol)
        self.reltol = float(reltol)
        self.mask = tuple(norm_mask) if norm_mask is not None else (True,) * len(self.y)
        self.dtmax = abs(t1 - t0) if dtmax is None else float(dtmax)
        self.dtmin = float(dtmin)
        self.maxiters = int(maxiters)
        stops = sorted({float(s) for s in tstops if self.tdir * (s - t0) > 0 and self.tdir * (t1 - s) > 0},
                       key=lambda s: self.tdir * s)
        self.stops = stops + [self.t1]
        self.on_stop = on_stop
        self.on_accept = on_accept
        self.replay = list(steps) if steps is not None else None
        self.record = record
        self.steps = []        # (t_n, h_n) of accepted steps
        self.stepdata = []     # (t_n, h_n, y_n, K) if record
        self.nf = 0
        self.naccept = 0
        self.nreject = 0
        self.retcode = RET_SUCCESS
        self.qold = T.QOLDINIT
        self.dt0 = float(dt0)

    # -- helpers ------------------------------------------------------------
    def _eval(self, y, t):
        self.nf += 1
        return tuple(np.asarray(k, dtype=np.float64) for k in self.F(y, t))

    def _initdt(self, k1):
        """Initial step: OrdinaryDiffEq's ode_determine_initdt (Hairer's algorithm)."""
        y0 = self.y
        sk = [self.abstol + np.abs(c) * self.reltol for c in y0]
        s0, n = _rms_sum([c / s for c, s in zip(y0, sk)], self.mask)
        s1, _ = _rms_sum([k / s for k, s in zip(k1, sk)], self.mask)
        d0 = math.sqrt(s0 / n)
        d1 = math.sqrt(s1 / n)
        smalldt = max(self.dtmin, 1e-6)
        if d0 < 1e-5 or d1 < 1e-5:
            dt0 = smalldt
        else:
            dt0 = 0.01 * (d0 / d1)
        dt0 = self._r(min(dt0, self.dtmax))
        y1 = tuple(c + self.tdir * dt0 * k for c, k in zip(y0, k1))
        f1 = self._eval(y1, self.t + self.tdir * dt0)
        s2, _ = _rms_sum([(a - b) / s for a, b, s in zip(f1, k1, sk)], self.mask)
        d2 = math.sqrt(s2 / n) / dt0
        m = max(d1, d2)
        if m <= 1e-15:
            dt1 = max(1e-6, dt0 * 1e-3)
        else:
            dt1 = 10.0 ** (-(2.0 + math.log10(m)) / T.ORDER)
        return self._r(max(self.dtmin, min(100.0 * dt0, dt1, self.dtmax)))

    def _stages(self, k1, h):
        y, t = self.y, self.t
        K = [k1]
        for i in range(1, 7):
            Yi = tuple(c + h * sum(T.A[i, j] * K[j][ci] for j in range(i)) for ci, c in enumerate(y))
            K.append(self._eval(Yi, t + T.C[i] * h))
            if i == 6:
                ynew = Yi
        return K, ynew

    def _eest(self, K, ynew, h):
        errs = []
        for ci, c in enumerate(self.y):
            if not self.mask[ci]:
                errs.append(None)
                continue
            ut = h * sum(T.BTILDE[j] * K[j][ci] for j in range(7))
            sc = self.abstol + np.maximum(np.abs(c), np.abs(ynew[ci])) * self.reltol
            errs.append(ut / sc)
        s, n = _rms_sum([e for e in errs if e is not None], [True] * sum(self.mask))
        return math.sqrt(s / n)

    def dense(self, t):
        """Forward dense output u(t) from recorded steps (record=True)."""
        ts = [d[0] for d in self.stepdata]
        if self.tdir > 0:
            i = max(0, bisect.bisect_right(ts, t) - 1)
        else:
            i = max(0, bisect.bisect_right([-x for x in ts], -t) - 1)
        tn, h, yn, K = self.stepdata[i]
        th = (t - tn) / h
        bw = T.interp_weights(th)
        return tuple(c + h * sum(bw[j] * K[j][ci] for j in range(7)) for ci, c in enumerate(yn))

    # -- main loop ------------------------------------------------------------
    def solve(self, on_save=None, saveat=()):
        """Integrate to t1. ``on_save(idx, y)`` receives the interpolated state at
        each ``saveat`` point (sorted in the direction of integration)."""
        saveat = list(saveat)
        isave = 0
        while isave < len(saveat) and saveat[isave] == self.t:
            on_save(isave, self.y)
            isave += 1
        k1 = self._eval(self.y, self.t)
        if self.replay is None:
            dt = self.dt0 if self.dt0 > 0 else self._initdt(k1)
        else:
            dt = None
        istop = 0
        it = 0
        while self.tdir * (self.t1 - self.t) > 0:
            if self.replay is not None:
                if it >= len(self.replay):
                    break
                tn, h = self.replay[it]
                assert abs(tn - self.t) <= 1e-12 * max(1.0, abs(tn)), (tn, self.t)
                tnext = self.replay[it + 1][0] if it + 1 < len(self.replay) else self.t1
                clipped = tnext == self.stops[istop]
            else:
                stop = self.stops[istop]
                rem = self._r(abs(stop - self.t))
                h = self.tdir * min(abs(dt), rem)
                clipped = abs(dt) >= rem
            if it >= self.maxiters:
                self.retcode = RET_MAXITERS
                break
            it += 1
            K, ynew = self._stages(k1, h)
            if self.replay is not None:
                EEst, accept = 0.0, True
            else:
                EEst = self._r(self._eest(K, ynew, h))
                if not math.isfinite(EEst):
                    self.retcode = RET_UNSTABLE
                    break
                accept = EEst <= 1.0
                if EEst == 0.0:
                    q = 1.0 / T.QMAX
                    q11 = 0.0
                else:
                    q11 = EEst ** T.BETA1
                    q = q11 / self.qold ** T.BETA2
                    q = max(1.0 / T.QMAX, min(1.0 / T.QMIN, q / T.GAMMA))
            if accept:
                tnew = self.stops[istop] if clipped else self._r(self.t + h)
                if self.record:
                    self.stepdata.append((self.t, h, self.y, K))
                self.steps.append((self.t, h))
                # saveat points in (t, tnew]
                while isave < len(saveat) and self.tdir * (saveat[isave] - tnew) <= 0:
                    s = saveat[isave]
                    if s == tnew:
                        on_save(isave, ynew)
                    else:
                        th = (s - self.t) / h
                        bw = T.interp_weights(th)
                        on_save(isave, tuple(c + h * sum(bw[j] * K[j][ci] for j in range(7))
                                             for ci, c in enumerate(self.y)))
                    isave += 1
                if self.on_accept is not None:
                    self.on_accept(self.t, h, self.y, K)
                self.y = ynew
                self.t = tnew
                self.naccept += 1
                k1 = K[6]
                if self.replay is None:
                    if T.QSTEADY_MIN <= q <= T.QSTEADY_MAX:
                        q = 1.0
                    self.qold = self._r(max(EEst, T.QOLDINIT))
                    dtnew = abs(h) / q
                    dtnew = min(self.dtmax, dtnew)
                    dtnew = max(dtnew, self.dtmin)
                    dt = self._r(dtnew)
                if clipped and istop < len(self.stops) - 1:
                    istop += 1
                    if self.on_stop is not None:
                        newy = self.on_stop(self.t, self.y)
                        if newy is not None:
                            self.y = tuple(np.array(c, dtype=np.float64) for c in newy)
                            k1 = self._eval(self.y, self.t)
                if not all(np.all(np.isfinite(c)) for c in self.y):
                    self.retcode = RET_UNSTABLE
                    break
            else:
                self.nreject += 1
                dt = self._r(abs(h) / min(1.0 / T.QMIN, q11 / T.GAMMA))
                if dt <= self.dtmin:
                    self.retcode = RET_DTMIN
                    break
        return self


# ---------------------------------------------------------------------------
# NeuralODE forward solve
# ---------------------------------------------------------------------------
def solve_forward(rhs, u0, t0, t1, saveat, abstol, reltol, dt0=0.0, maxiters=100000,
                  steps=None, record=True, dtmin=0.0, time_f32=False):
    """Forward solve; returns (usave [S,B,nsave], integrator)."""
    u0 = np.asarray(u0, dtype=np.float64)
    saveat = [float(s) for s in saveat]
    out = np.zeros(u0.shape + (len(saveat),))

    def on_save(i, y):
        out[..., i] = y[0]

    integ = Tsit5(lambda y, t: (rhs.f(y[0], t),), (u0,), t0, t1, abstol, reltol, dt0=dt0,
                  maxiters=maxiters, steps=steps, record=record, dtmin=dtmin, time_f32=time_f32)
    integ.solve(on_save=on_save, saveat=saveat)
    return out, integ


# ---------------------------------------------------------------------------
# Adjoints
# ---------------------------------------------------------------------------
def _backward_stops(saveat, t0):
    s = sorted(set(float(x) for x in saveat), reverse=True)
    return s


def adjoint_interpolating(rhs, fwd, saveat, dL_dusave, t0, abstol, reltol, maxiters=100000,
                          time_f32=False):
    """InterpolatingAdjoint: backward solve of (lam, mu) with u(t) from the
    forward dense output. Returns (dL/du0, dL/dp, integrator)."""
    saveat = [float(s) for s in saveat]
    idx = {}
    for i, s in enumerate(saveat):
        idx.setdefault(s, []).append(i)
    stops = _backward_stops(saveat, t0)
    t_last = stops[0]
    lam0 = sum(dL_dusave[..., i] for i in idx[t_last])
    P = rhs.nparams()

    def F(y, t):
        u = fwd.dense(t)[0]
        gu, gp = rhs.vjp(u, t, y[0])
        return (-gu, -gp)

    def on_stop(t, y):
        if t in idx:
            return (y[0] + sum(dL_dusave[..., i] for i in idx[t]), y[1])
        return None

    integ = Tsit5(F, (lam0, np.zeros(P)), t_last, t0, abstol, reltol, norm_mask=(True, False),
                  tstops=stops[1:], on_stop=on_stop, maxiters=maxiters, time_f32=time_f32)
    if t_last > t0:
        integ.solve()
    lam, mu = integ.y
    if t0 in idx and t_last > t0:
        pass  # jump at t0 applied by on_stop (t0 is the final stop)
    if t_last == t0:
        lam = lam0
    # the final stop t0 is the end of the span: on_stop is not called there
    if t0 in idx and t_last > t0:
        lam = lam + sum(dL_dusave[..., i] for i in idx[t0])
    return lam, mu, integ


def adjoint_gauss(rhs, fwd, saveat, dL_dusave, t0, abstol, reltol, npts=4, maxiters=100000):
    """Quadrature adjoint (QuadratureAdjoint / GaussAdjoint, re-exported at
    src/DiffEqFlux.jl:53): the backward solve carries lam only (same
    tableau, controller and lam-norm as InterpolatingAdjoint), and
    dL/dp = int_{t0}^{T} lam^T df/dp dt is integrated by ``npts``-point
    Gauss-Legendre over every accepted adjoint step, with lam(theta) from that
    step's free interpolant and u from the forward dense output. Returns
    (dL/du0, dL/dp, integrator)."""
    saveat = [float(s) for s in saveat]
    idx = {}
    for i, s in enumerate(saveat):
        idx.setdefault(s, []).append(i)
    stops = _backward_stops(saveat, t0)
    t_last = stops[0]
    lam0 = sum(dL_dusave[..., i] for i in idx[t_last])
    mu = np.zeros(rhs.nparams())
    xg, wg = np.polynomial.legendre.leggauss(npts)
    thetas, weights = (xg + 1.0) / 2.0, wg / 2.0

    def F(y, t):
        u = fwd.dense(t)[0]
        gu, _ = rhs.vjp(u, t, y[0])
        return (-gu,)

    def on_stop(t, y):
        if t in idx:
            return (y[0] + sum(dL_dusave[..., i] for i in idx[t]),)
        return None

    def on_accept(t, h, y, K):
        for th, w in zip(thetas, weights):
            bw = T.interp_weights(th)
            lam = y[0] + h * sum(bw[j] * K[j][0] for j in range(7))
            tg = t + th * h
            u = fwd.dense(tg)[0]
            _, gp = rhs.vjp(u, tg, lam)
            mu[:] += w * abs(h) * gp

    integ = Tsit5(F, (lam0,), t_last, t0, abstol, reltol, tstops=stops[1:], on_stop=on_stop,
                  maxiters=maxiters, on_accept=on_accept)
    if t_last > t0:
        integ.solve()
    lam = integ.y[0] if t_last > t0 else lam0
    if t0 in idx and t_last > t0:
        lam = lam + sum(dL_dusave[..., i] for i in idx[t0])
    return lam, mu, integ


def adjoint_backsolve(rhs, usave, saveat, dL_dusave, t0, abstol, reltol, maxiters=100000):
    """BacksolveAdjoint (checkpointing on): co-integrate u backwards with (lam, mu),
    reset u to the saved forward value at each save point."""
    saveat = [float(s) for s in saveat]
    idx = {}
    for i, s in enumerate(saveat):
        idx.setdefault(s, []).append(i)
    stops = _backward_stops(saveat, t0)
    t_last = stops[0]
    lam0 = sum(dL_dusave[..., i] for i in idx[t_last])
    u_last = usave[..., idx[t_last][0]]
    P = rhs.nparams()

    def F(y, t):
        fu = rhs.f(y[0], t)
        gu, gp = rhs.vjp(y[0], t, y[1])
        return (fu, -gu, -gp)

    def on_stop(t, y):
        if t in idx:
            return (usave[..., idx[t][0]], y[1] + sum(dL_dusave[..., i] for i in idx[t]), y[2])
        return None

    integ = Tsit5(F, (u_last, lam0, np.zeros(P)), t_last, t0, abstol, reltol,
                  norm_mask=(True, True, False), tstops=stops[1:], on_stop=on_stop, maxiters=maxiters)
    if t_last > t0:
        integ.solve()
    u, lam, mu = integ.y
    if t_last == t0:
        lam = lam0
    if t0 in idx and t_last > t0:
        lam = lam + sum(dL_dusave[..., i] for i in idx[t0])
    return lam, mu, integ
