"""Oracle package: CPU restatement of the reference FM-DBZP acquisition path.

Test infrastructure only. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` import it, as the checker; the product never does.
"""
