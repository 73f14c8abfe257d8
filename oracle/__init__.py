"""CPU oracle for the GB300 neural-ODE kernels (test infrastructure only).

Nothing in the product imports this package: only the tests, the smoke check
and the CPU-baseline leg of the benchmark use it, as the checker.
"""
