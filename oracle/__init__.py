"""CPU oracle of the polarisation path: test infrastructure only.

Imported by tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` -- never by the ``muspinsim_gb300`` package itself.
"""
