"""CPU oracle for the batched SCF path (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this package.  The product path (``pyseqm_gb300``) never calls it.
"""
