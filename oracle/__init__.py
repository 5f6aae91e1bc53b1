"""CPU oracle for the exact-diagonalization hot path — TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy/SciPy, the algorithms of impurityModel's
``impurityModel/ed/finite.py`` and ``impurityModel/ed/spectra.py`` that the GPU engine
replaces.  It is the checker: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` import it.  The product package ``impuritymodel_gb300``
never imports it and has no CPU fallback.

Parity of the oracle itself is pinned against the upstream implementation: fixtures in
``tests/golden/`` were produced by running upstream (``tests/golden/make_golden.py``)
and ``tests/test_oracle_golden.py`` checks the oracle against them.
"""

from .ed_oracle import *  # noqa: F401,F403
