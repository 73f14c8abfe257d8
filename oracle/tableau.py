"""Tsit5 tableau, free interpolant and PI-controller constants (FP64).

TEST INFRASTRUCTURE ONLY. This module belongs to the CPU oracle that checks the
CUDA kernels; no product code path imports it.

Source of the numbers
---------------------
The reference (DiffEqFlux.jl) does not hold the integrator: `NeuralODE` calls
`solve(prob, n.args...; ...)` (src/neural_de.jl:55-58) and its tests pass
`Tsit5()` as the algorithm (test/BasicNeuralDE/neural_de_tests.jl:43). Tsit5
lives in OrdinaryDiffEq (compat "7", Project.toml:57), which is not vendored.
The coefficients below restate the published method:

  Ch. Tsitouras, "Runge-Kutta pairs of order 5(4) satisfying only the first
  column simplifying assumption", Comput. Math. Appl. 62 (2011) 770-775,

with the error weights written as ``btilde = b - bhat`` and the free 4th-order
dense output ``b_i(theta)`` written as polynomials in theta. They are pinned by
the order conditions in ``oracle/check_tableau.py`` (5th order for ``b``, 4th
order for ``bhat``, 4th order for ``b(theta)`` at every theta), which the CPU
test-suite runs.

The PI step-size controller constants are the documented defaults of the
integrator for a 5th-order explicit method (beta1 = 7/(10*5), beta2 =
2/(5*5), qmin = 1/5, qmax = 10, gamma = 9/10, qoldinit = 1e-4); they cannot
be observed here without a Julia runtime and are recorded as assumptions.
"""
import numpy as np

NSTAGES = 7
ORDER = 5

C = np.array([0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0])

A = np.zeros((7, 7))
A[1, 0] = 0.161
A[2, 0] = -0.008480655492356989
A[2, 1] = 0.335480655492357
A[3, 0] = 2.897153057105493
A[3, 1] = -6.359448489975075
A[3, 2] = 4.3622954328695815
A[4, 0] = 5.325864828439257
A[4, 1] = -11.748883564062828
A[4, 2] = 7.4955393428898365
A[4, 3] = -0.09249506636175525
A[5, 0] = 5.86145544294642
A[5, 1] = -12.92096931784711
A[5, 2] = 8.159367898576159
A[5, 3] = -0.071584973281401
A[5, 4] = -0.028269050394068383
A[6, 0] = 0.09646076681806523
A[6, 1] = 0.01
A[6, 2] = 0.4798896504144996
A[6, 3] = 1.379008574103742
A[6, 4] = -3.290069515436081
A[6, 5] = 2.324710524099774

# FSAL: the 5th-order weights are the last row of A, b7 = 0.
B = A[6].copy()

# btilde = b - bhat (embedded 4th-order pair)
BTILDE = np.array([
    -0.00178001105222577714,
    -0.0008164344596567469,
    0.007880878010261995,
    -0.1447110071732629,
    0.5823571654525552,
    -0.45808210592918697,
    1.0 / 66.0,
])

# Dense output: b_i(theta) = sum_m R[i, m] * theta^(m+1), m = 0..3
R = np.array([
    [1.0, -2.763706197274826, 2.9132554618219126, -1.0530884977290216],
    [0.0, 0.13169999999999998, -0.2234, 0.1017],
    [0.0, 3.9302962368947516, -5.941033872131505, 2.490627285651253],
    [0.0, -12.411077166933676, 30.33818863028232, -16.548102889244902],
    [0.0, 37.50931341651104, -88.1789048947664, 47.37952196281928],
    [0.0, -27.896526289197286, 65.09189467479366, -34.87065786149661],
    [0.0, 1.5, -4.0, 2.5],
])

# PI controller (documented defaults for a 5th-order explicit RK method)
BETA1 = 7.0 / 50.0
BETA2 = 2.0 / 25.0
QMIN = 1.0 / 5.0
QMAX = 10.0
GAMMA = 9.0 / 10.0
QOLDINIT = 1.0e-4
QSTEADY_MIN = 1.0
QSTEADY_MAX = 1.0


def interp_weights(theta):
    """b_i(theta), i = 1..7, for the free 4th-order Tsit5 interpolant."""
    th = float(theta)
    pw = np.array([th, th * th, th ** 3, th ** 4])
    return R @ pw
