"""CPU oracle for the generalized-winding-number path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference arm may import this package.  The product library never does.
"""
