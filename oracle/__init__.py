"""CPU oracle for the KinectFusion per-frame path -- test infrastructure only.

Imported by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg as
the checker.  The product package never imports anything from here.
"""
