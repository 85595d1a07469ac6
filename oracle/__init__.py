"""Checker for the matched-filter hot path.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, by ``__graft_entry__.smoke``
and by ``bench.py``'s CPU-baseline leg.  The product package
``fast_matched_filter_gb300`` never imports it.

* ``oracle.cpu``  -- ctypes front-end over ``fmf_oracle.c`` (a C restatement
  of the reference CPU library) and, when it was built, over the reference
  library itself compiled from its own source into ``oracle/_ref``.
* ``oracle.fp64`` -- an FP64 numpy evaluation of the same formulas, used to
  state the error of every FP32/BF16 form.
"""
