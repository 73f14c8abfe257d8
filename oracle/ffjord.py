"""FP64 restatement of the FFJORD right-hand side and its adjoint VJP (test
infrastructure only).

Follows src/ffjord.jl:
  * augmented state [z; delta_logp], zero-initialised delta_logp rows (:149-153);
  * RHS  [f(z); -trace(df/dz)] (:81-136), with the trace either exact
    (monte_carlo = false, :120-129) or the Hutchinson estimate e^T (df/dz) e
    (monte_carlo = true, :92-115);
  * logpx = logpz(z(t1)) - delta_logp(t1) with the standard-normal base
    logpz = -|z|^2/2 - d/2 log(2 pi) (:171-176);
  * regularize = true (:131-132, :151-168): two more rows integrate |f|^2
    (sum over the d outputs) and |e^T J| (the 2-norm of the vector-Jacobian
    product along the noise e; the exact-trace mode draws e for this row
    only).
Deliberate, documented differences: the noise e is drawn once per sample per
solve (Rademacher or Gaussian) instead of fresh on every RHS call, so that
the ODE -- and its adjoint -- is well defined; e^T J e is evaluated as e . (J e)
(a forward-mode directional derivative) rather than (e^T J) . e (a reverse
pass); the two are the same number.

The adjoint needs d/d(z, p) of e^T J e: reverse mode over the forward-mode
tangent computation ("reverse over forward"), written out per layer below.
For the |e^T J| row: with v = J^T e and w = v / |v|, d|v| = w^T dv =
e^T (dJ) w, so its cotangent is that of e^T J w with w held fixed -- the same
reverse-over-forward pass along the direction w, with e as the weight.
"""
import numpy as np

try:
    from . import mlp as omlp
except ImportError:  # pragma: no cover
    import mlp as omlp  # type: ignore


def _d1(code, a, z):
    if code == omlp.ACT_TANH:
        return 1.0 - a * a
    if code == omlp.ACT_SOFTPLUS:
        return 1.0 / (1.0 + np.exp(-z))
    return np.ones_like(a)


def _d2(code, a, z):
    if code == omlp.ACT_TANH:
        return -2.0 * a * (1.0 - a * a)
    if code == omlp.ACT_SOFTPLUS:
        s = 1.0 / (1.0 + np.exp(-z))
        return s * (1.0 - s)
    return np.zeros_like(a)


class FFJORDRHS:
    """RHS of the augmented FFJORD state y = [z (d x B); delta_logp (1 x B)]."""

    def __init__(self, mlp, p, noise=None, exact=False, regularize=False):
        assert not mlp.cube_input
        assert not regularize or noise is not None, "the |e^T J| row needs the noise e"
        self.mlp = mlp
        self.p = np.asarray(p, dtype=np.float64)
        self.noise = noise
        self.exact = exact
        self.regularize = regularize
        self.d = mlp.state_dim
        self.nf = 0

    def nparams(self):
        return self.mlp.nparams()

    def _input(self, z, t):
        if self.mlp.time_input:
            return np.vstack([z, np.full((1, z.shape[1]), t)])
        return z

    def _fwd_tangent(self, z, t, e):
        """Primal activations and tangents along e: lists of (z_l, a_l, zdot_l, adot_l)."""
        layers = self.mlp.unflatten(self.p)
        a = self._input(z, t)
        adot = np.vstack([e, np.zeros((a.shape[0] - e.shape[0], e.shape[1]))])
        cache = [(None, a, None, adot)]
        for l, (W, b) in enumerate(layers):
            zl = W @ a + b[:, None]
            zd = W @ adot
            a = omlp._act(self.mlp.acts[l], zl)
            adot = _d1(self.mlp.acts[l], a, zl) * zd
            cache.append((zl, a, zd, adot))
        return cache

    def _trace(self, z, t):
        if self.exact:
            tr = np.zeros((1, z.shape[1]))
            f = None
            for i in range(self.d):
                e = np.zeros_like(z)
                e[i] = 1.0
                c = self._fwd_tangent(z, t, e)
                f = c[-1][1]
                tr[0] += c[-1][3][i]
            return f, tr
        c = self._fwd_tangent(z, t, self.noise)
        return c[-1][1], np.sum(self.noise * c[-1][3], axis=0, keepdims=True)

    def _vjp_input(self, z, t, g):
        """J^T g: the cotangent of the chain input (z rows only) for the output
        cotangent g, by a plain reverse pass."""
        layers = self.mlp.unflatten(self.p)
        a = self._input(z, t)
        acts = [a]
        for l, (W, b) in enumerate(layers):
            a = omlp._act(self.mlp.acts[l], W @ a + b[:, None])
            acts.append(a)
        for l in range(len(layers) - 1, -1, -1):
            zl = layers[l][0] @ acts[l] + layers[l][1][:, None]
            g = layers[l][0].T @ (g * _d1(self.mlp.acts[l], acts[l + 1], zl))
        return g[: self.d]

    def f(self, y, t):
        self.nf += 1
        z = y[: self.d]
        f, tr = self._trace(z, t)
        if not self.regularize:
            return np.vstack([f, -tr])
        v = self._vjp_input(z, t, self.noise)
        return np.vstack([f, -tr, np.sum(f * f, axis=0, keepdims=True),
                          np.sqrt(np.sum(v * v, axis=0, keepdims=True))])

    def vjp(self, y, t, lam):
        """(lam^T dg/dy, lam^T dg/dp) for g = [f; -e^T J e] (Hutchinson) or
        g = [f; -tr J] (exact)."""
        z = y[: self.d]
        lz, ll = lam[: self.d], lam[self.d:self.d + 1]
        layers = self.mlp.unflatten(self.p)
        # (tangent direction, weight of the tangent output) per pass
        es = [(self.noise, -ll * self.noise)] if not self.exact else []
        if self.exact:
            for i in range(self.d):
                e = np.zeros_like(z)
                e[i] = 1.0
                es.append((e, -ll * e))
        if self.regularize:
            # |f|^2 row: cotangent 2 lam f on the primal output
            f = self._fwd_tangent(z, t, np.zeros_like(z))[-1][1]
            lz = lz + 2.0 * lam[self.d + 1:self.d + 2] * f
            # |e^T J| row: direction w = v/|v|, weight lam e
            v = self._vjp_input(z, t, self.noise)
            nv = np.sqrt(np.sum(v * v, axis=0, keepdims=True))
            w = np.divide(v, nv, out=np.zeros_like(v), where=nv > 0)
            es.append((w, lam[self.d + 2:self.d + 3] * self.noise))
        gz_tot = np.zeros_like(z)
        grads_tot = None
        for k, (e, adbar) in enumerate(es):
            c = self._fwd_tangent(z, t, e)
            abar = lz if k == 0 else np.zeros_like(lz)   # primal cotangent (f appears once)
            grads = [None] * len(layers)
            for l in range(len(layers) - 1, -1, -1):
                zl, al, zd, _ = c[l + 1]
                a_in, adot_in = c[l][1], c[l][3]
                code = self.mlp.acts[l]
                d1 = _d1(code, al, zl)
                d2 = _d2(code, al, zl)
                zdbar = adbar * d1
                zbar = adbar * d2 * zd + abar * d1
                W = layers[l][0]
                gW = zbar @ a_in.T + zdbar @ adot_in.T
                grads[l] = (gW, zbar.sum(axis=1))
                abar = W.T @ zbar
                adbar = W.T @ zdbar
            g = self.mlp.flatten(grads)
            grads_tot = g if grads_tot is None else grads_tot + g
            gz_tot += abar[: self.d]
        return np.vstack([gz_tot, np.zeros_like(lam[self.d:])]), grads_tot


def logpx_from_final(yT, d):
    """logpx = logpz(z) - delta_logp with the standard normal base (src/ffjord.jl:171-176)."""
    z = yT[:d]
    logpz = -0.5 * np.sum(z * z, axis=0) - 0.5 * d * np.log(2.0 * np.pi)
    return logpz - yT[d]
