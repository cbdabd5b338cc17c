"""CPU oracle for the bonded-DEM Newton path (test infrastructure, not product).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this package, and only as the checker.  The product
path (``dpf_gb300``) never calls it and raises if its CUDA library is missing.

Pinning: the restatement in :mod:`oracle.dem` is checked against golden
vectors produced by running the reference's own Python code
(``tests/golden/make_golden.py``), so parity is pinned, not self-referential.
"""
