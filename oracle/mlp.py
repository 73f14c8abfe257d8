"""FP64 multilayer-perceptron right-hand side with its vector-Jacobian product.

TEST INFRASTRUCTURE ONLY (part of the CPU oracle).

Restates the Lux model the reference solves: ``dudt(u, p, t) = model(u, p)``
(src/neural_de.jl:50) with ``model = Chain([x -> x.^3,] Dense(d0, d1, act), ...)``
(docs/src/examples/neural_ode.md:32, test/BasicNeuralDE/neural_de_tests.jl:17).
A Lux ``Dense(in, out, act)`` computes ``act.(W * x .+ b)`` with ``W`` of shape
``out x in``; the last layer of the configurations here has no activation.

Parameter layout (the drop-in boundary): the flat vector that
``ComponentArray(ps)`` produces, i.e. for each layer in order its weight
(``out x in``, column-major) followed by its bias (``out``).

The state is a matrix ``S x B`` (one column per trajectory), exactly as the
reference passes ``x`` to ``ODEProblem`` (src/neural_de.jl:52).
"""
import numpy as np

ACT_IDENTITY = 0
ACT_TANH = 1
ACT_SOFTPLUS = 2

_ACT_NAMES = {"identity": ACT_IDENTITY, "tanh": ACT_TANH, "softplus": ACT_SOFTPLUS}


def act_code(a):
    return _ACT_NAMES[a] if isinstance(a, str) else int(a)


def _act(code, z):
    if code == ACT_TANH:
        return np.tanh(z)
    if code == ACT_SOFTPLUS:
        return np.logaddexp(0.0, z)
    return z


def _dact_from_out(code, a, z):
    """act'(z), written in terms of the output where that is exact."""
    if code == ACT_TANH:
        return 1.0 - a * a
    if code == ACT_SOFTPLUS:
        return 1.0 / (1.0 + np.exp(-z))
    return np.ones_like(a)


class MLP:
    """Chain([cube,] Dense(d0,d1,act1), ..., Dense(d_{L-1}, d_L, act_L))."""

    def __init__(self, dims, acts, cube_input=False, time_input=False):
        assert len(acts) == len(dims) - 1
        self.dims = [int(d) for d in dims]
        self.acts = [act_code(a) for a in acts]
        self.cube_input = bool(cube_input)
        self.time_input = bool(time_input)
        self.state_dim = self.dims[0] - (1 if self.time_input else 0)
        assert self.dims[-1] == self.state_dim
        self.nlayers = len(acts)

    # ---- parameter layout -------------------------------------------------
    def nparams(self):
        return sum(self.dims[l] * self.dims[l + 1] + self.dims[l + 1] for l in range(self.nlayers))

    def unflatten(self, p):
        p = np.asarray(p, dtype=np.float64)
        assert p.size == self.nparams()
        out, o = [], 0
        for l in range(self.nlayers):
            din, dout = self.dims[l], self.dims[l + 1]
            W = p[o:o + din * dout].reshape(din, dout).T  # column-major out x in
            o += din * dout
            b = p[o:o + dout]
            o += dout
            out.append((W, b))
        return out

    def flatten(self, layers):
        parts = []
        for (W, b) in layers:
            parts.append(np.asarray(W, dtype=np.float64).T.reshape(-1))
            parts.append(np.asarray(b, dtype=np.float64).reshape(-1))
        return np.concatenate(parts)

    def glorot_uniform(self, rng, dtype=np.float32):
        """Glorot-uniform weights and zero biases, flat in the Lux order."""
        layers = []
        for l in range(self.nlayers):
            din, dout = self.dims[l], self.dims[l + 1]
            lim = np.sqrt(6.0 / (din + dout))
            W = rng.uniform(-lim, lim, size=(dout, din))
            b = np.zeros(dout)
            layers.append((W, b))
        return self.flatten(layers).astype(dtype)

    # ---- evaluation -------------------------------------------------------
    def _input(self, u, t):
        x = u ** 3 if self.cube_input else u
        if self.time_input:
            x = np.vstack([x, np.full((1, u.shape[1]), t)])
        return x

    def forward(self, p, u, t=0.0, keep=False):
        layers = self.unflatten(p)
        a = self._input(np.asarray(u, dtype=np.float64), t)
        cache = [(None, a)]
        for l, (W, b) in enumerate(layers):
            z = W @ a + b[:, None]
            a = _act(self.acts[l], z)
            cache.append((z, a))
        return (a, cache) if keep else a

    def vjp(self, p, u, t, lam):
        """(lam^T df/du, lam^T df/dp summed over the batch)."""
        layers = self.unflatten(p)
        y, cache = self.forward(p, u, t, keep=True)
        g = np.asarray(lam, dtype=np.float64)
        grads = [None] * self.nlayers
        for l in range(self.nlayers - 1, -1, -1):
            z, a = cache[l + 1]
            g = g * _dact_from_out(self.acts[l], a, z)
            a_in = cache[l][1]
            grads[l] = (g @ a_in.T, g.sum(axis=1))
            g = layers[l][0].T @ g
        if self.time_input:
            g = g[:self.state_dim]
        if self.cube_input:
            g = g * 3.0 * np.asarray(u, dtype=np.float64) ** 2
        return g, self.flatten(grads)


class MLPRHS:
    """ODE right-hand side ``f(u, p, t) = model(u, p)`` bound to flat parameters."""

    def __init__(self, mlp, p):
        self.mlp = mlp
        self.p = np.asarray(p, dtype=np.float64)
        self.nf = 0
        self.nvjp = 0

    def f(self, u, t):
        self.nf += 1
        return self.mlp.forward(self.p, u, t)

    def vjp(self, u, t, lam):
        self.nvjp += 1
        return self.mlp.vjp(self.p, u, t, lam)

    def nparams(self):
        return self.mlp.nparams()
