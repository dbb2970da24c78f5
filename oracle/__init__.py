"""Test oracle for pyiid_gb300 (FP64 restatements of the reference path).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``; never by the ``pyiid_gb300`` package.
"""
