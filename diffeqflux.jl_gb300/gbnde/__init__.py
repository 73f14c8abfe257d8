"""gbnde -- GB300-native neural differential equations (host package).

Python host side of libgbnde.so, mirroring the DiffEqFlux layer API:
``NeuralODE`` (src/neural_de.jl), ``FFJORD`` (src/ffjord.jl) and
``multiple_shoot`` (src/multiple_shooting.jl), with the sensealg markers the
reference re-exports (src/DiffEqFlux.jl:53-56).
"""
from ._lib import GbndeError, load  # noqa: F401
from .layers import (  # noqa: F401
    Array, BacksolveAdjoint, Chain, Dense, GaussAdjoint, GB300Tsit5, InterpolatingAdjoint, NeuralODE,
    QuadratureAdjoint,
    ODESolution, Solver, Tsit5, WrappedFunction, ZygoteVJP, cube,
)
from .ffjord import FFJORD, FFJORDDistribution  # noqa: F401
from .layers import AugmentedNDELayer, DimMover  # noqa: F401
from .multiple_shooting import (group_ranges, mse_loss, multiple_shoot, multiple_shoot_batch,  # noqa: F401
                                sse_loss)
