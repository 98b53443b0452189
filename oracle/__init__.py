"""CPU oracle for the projection hot path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker.
"""
from .oracle import Oracle, OracleInput, load  # noqa: F401
