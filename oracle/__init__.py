"""Gaussian-atom Radon oracle package: test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it.  The product package never imports it.
"""
