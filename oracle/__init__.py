"""Oracle: CPU FP64 restatement of the reference's inference path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this package; the product path never does.
"""
