"""Pins the Tsit5 tableau in ``oracle/tableau.py`` by the Runge-Kutta order conditions.

TEST INFRASTRUCTURE ONLY (part of the CPU oracle).

The tableau restates Tsitouras (2011); no golden vectors for it exist in the
reference (which only calls ``solve(prob, Tsit5())``, src/neural_de.jl:55-58),
so the pin is mathematical: every rooted tree up to order 5 for ``b``, up to
order 4 for ``bhat = b - btilde`` and for the dense output ``b(theta)`` (with
right-hand side ``theta^rho / gamma``), and the row-sum condition ``c = A 1``.
Running this file prints the worst residual and exits non-zero above 1e-12.
"""
import sys

import numpy as np

try:
    from . import tableau as T
except ImportError:  # run as a script
    import tableau as T  # type: ignore


def _trees(A, c):
    """(order, gamma, Phi) for the 17 rooted trees of order <= 5."""
    Ac = A @ c
    Ac2 = A @ (c ** 2)
    AAc = A @ Ac
    return [
        (1, 1.0, np.ones_like(c)),
        (2, 2.0, c),
        (3, 3.0, c ** 2),
        (3, 6.0, Ac),
        (4, 4.0, c ** 3),
        (4, 8.0, c * Ac),
        (4, 12.0, Ac2),
        (4, 24.0, AAc),
        (5, 5.0, c ** 4),
        (5, 10.0, c ** 2 * Ac),
        (5, 15.0, c * Ac2),
        (5, 30.0, c * AAc),
        (5, 20.0, Ac ** 2),
        (5, 20.0, A @ (c ** 3)),
        (5, 40.0, A @ (c * Ac)),
        (5, 60.0, A @ Ac2),
        (5, 120.0, A @ AAc),
    ]


def residuals():
    A, c, b = T.A, T.C, T.B
    bhat = b - T.BTILDE
    out = {}
    out["row_sum"] = float(np.max(np.abs(A.sum(axis=1) - c)))
    out["b_order5"] = max(abs(b @ phi - 1.0 / g) for (o, g, phi) in _trees(A, c))
    out["bhat_order4"] = max(abs(bhat @ phi - 1.0 / g) for (o, g, phi) in _trees(A, c) if o <= 4)
    # bhat must NOT be 5th order (otherwise the error estimate would vanish)
    out["bhat_not_order5"] = max(abs(bhat @ phi - 1.0 / g) for (o, g, phi) in _trees(A, c) if o == 5)
    worst = 0.0
    for th in np.linspace(0.0, 1.0, 41):
        bt = T.interp_weights(th)
        for (o, g, phi) in _trees(A, c):
            if o <= 4:
                worst = max(worst, abs(bt @ phi - th ** o / g))
    out["dense_order4"] = worst
    out["dense_at_1_equals_b"] = float(np.max(np.abs(T.interp_weights(1.0) - b)))
    out["btilde_sum"] = abs(float(T.BTILDE.sum()))
    return out


def main():
    r = residuals()
    for k, v in r.items():
        print(f"{k:22s} {v:.3e}")
    ok = all(v < 1e-12 for k, v in r.items() if k != "bhat_not_order5") and r["bhat_not_order5"] > 1e-6
    print("tableau pinned" if ok else "TABLEAU CHECK FAILED")
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
