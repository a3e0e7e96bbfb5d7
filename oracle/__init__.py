"""Oracle package: CPU restatement of the reference hot path (test infrastructure only).

Imported only by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline / reference arm, always as the checker or the timed CPU baseline.
"""
