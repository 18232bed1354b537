"""CPU oracle for the efficient-filter-flow (EFF) path.

Test infrastructure only: ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it as the
checker or as the timed CPU baseline.  The product (``vmbd_gb300``) never
imports it.
"""
