"""Oracle: CPU restatement of the reference's hot path, used only as a checker.

Test infrastructure only.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference legs of ``bench.py`` may import this package; the
product (``rigidmultiblobswall_gb300``) never does.
"""
