"""CPU oracle for the pseudo-spectral solver step (test infrastructure only).

Nothing in the product imports this package. Only the tests, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and only as a
checker or as the timed CPU baseline.
"""
