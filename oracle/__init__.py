"""CPU oracle for the pypde spectral-Galerkin time-step path.

TEST INFRASTRUCTURE ONLY.  This package is a float64 NumPy restatement of the
reference algorithm (pypde by preiter93) used to check the CUDA path.  Only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it, and there only as the reference results are compared
against or as the timed CPU baseline.  The product package ``pypde_gb300`` never imports it and has no CPU
fallback.

Every function names the reference file:line it restates.  The oracle is
pinned against golden vectors produced by the reference itself
(``tests/golden/make_golden.py``) and against the reference's own
known-answer tests.

Modules
-------
spectral  DCT-I, Chebyshev / Shen bases, stencils, derivative recurrence
linalg    TDMA (offset k), FDMA, TwoDMA, FDMA type-2 (Poisson) sweeps
field     2-D transforms with 3/2 dealiasing, grad, convective term, averages
solver    ADI Helmholtz and fast-diagonalised Poisson plans
kernels.c the banded sweeps and the derivative recurrence in C (same operations,
          same order, no FMA contraction: bit-equal to the NumPy loops), loaded
          by _ck when built; without it the NumPy loops run
rbc2d     Rayleigh-Benard IMEX step, Nusselt numbers, kinetic energy
"""
from . import spectral, linalg, field, solver, rbc2d  # noqa: F401
