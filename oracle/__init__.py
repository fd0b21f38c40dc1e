"""ORACLE — test infrastructure, not product code.

A CPU, float64 restatement of BoTorch 0.18.1's GP-posterior + Monte-Carlo
acquisition path (SingleTaskGP.posterior -> qExpectedImprovement /
qLogNoisyExpectedImprovement value and gradient), written from the reference
sources and from the published algorithms of its two external dependencies
(gpytorch >= 1.15.2 and linear_operator >= 0.6.1, which are not vendored in
the reference tree; see ``oracle/gp.py`` for the parts restated from them).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU
baseline and ``--impl reference`` arm) may import this package, and only as
the checker or as the timed CPU baseline. The product package
``botorch_gb300`` never imports it: its compute path is the CUDA library and
it raises if that library is missing.

Pinning: the safe-math reductions and the Sobol normal base samples are pinned
bit-for-bit (or to 1 ulp) against golden vectors produced by importing the
reference's own modules (``tests/golden/make_golden.py``). The GP posterior
arithmetic lives in gpytorch/linear_operator, which cannot be imported in this
environment; there the oracle is pinned by the reference's own property and
differential tests (known qEI answers on fixed samples, LogEI bounds, cached
vs. uncached root decomposition) restated in ``tests/test_oracle.py``.
"""

from oracle import safe_math, sampling, gp, acquisition  # noqa: F401
