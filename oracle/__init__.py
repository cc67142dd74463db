"""FP64 CPU oracle for the EMSolvers time loops.

ORACLE / TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline legs of ``bench.py`` import this package, as the checker.
The product library (``emsolvers_gb300``) never imports or links it.
"""
from .oracle import *  # noqa: F401,F403
