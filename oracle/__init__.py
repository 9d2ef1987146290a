"""CPU oracle for the Schur-block Liouvillian hot path (TEST INFRASTRUCTURE ONLY).

This package restates, on the CPU, the algorithms of PermutationalInvariantDynamics.jl
that the GPU library replaces.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it, and only as the
checker or the timed CPU baseline.  The product path never calls into this package.
"""
