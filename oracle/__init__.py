"""Oracle: test infrastructure only.

A plain FP64 CPU restatement of the godunov_mhd_ct MUSCL-Hancock + CT stage (C++, in
``oracle_step.cpp`` / ``oracle_models.h``) and, where the reference tree is present, a bridge to
the reference's own per-cell math (``refkat/``). Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg import this package; the product never does.
"""
