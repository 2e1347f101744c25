"""ORACLE -- test infrastructure only.

CPU restatements of the reference algorithm, used as the checker by
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py``.  Nothing in ``zandpack_gb300`` imports this package.
"""
