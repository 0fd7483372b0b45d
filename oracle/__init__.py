"""CPU oracle for the DTO permutation path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline and
reference legs may import this package.  The product package never does.
"""
