"""CPU oracle for the convolutional gridding path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.  It is the checker, never the thing
measured as the GPU product and never a fallback for it.
"""
