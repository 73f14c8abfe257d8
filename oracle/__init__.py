"""CPU oracle for the GB300 neural-ODE kernels (test infrastructure only).

Nothing in the product imports this package: only the tests, the smoke check
and the CPU leg of the benchmark use it, to check and to time against.
"""
