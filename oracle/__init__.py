"""CPU oracle for the dense ampcor offset estimator (TEST INFRASTRUCTURE ONLY).

This package restates, in FP64 NumPy, the algorithm of ISCE2's PyCuAmpcor
(``contrib/PyCuAmpcor/src``) including its quirks.  It is the checker that the
CUDA path is compared against.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it; the product path
(``isce2_gb300``) never does, and never falls back to it.

Parity pins: the reference ships no tests, golden vectors or fixtures for this
path, so the oracle is pinned by known-answer tests (exact integer shifts,
constant fields, analytic sub-pixel shifts) and by committed golden vectors it
generates (``tests/golden``), not by outputs of the reference binary.
"""
