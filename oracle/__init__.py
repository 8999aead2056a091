"""Test infrastructure: the oracle for the MassiveMDS likelihood/gradient sweep.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this package, and only as the checker. The CUDA engine in ``massivemds_gb300``
never calls it.

* :func:`sum_of_increments`, :func:`gradient` - ctypes bindings to the C
  restatement in ``oracle/mds_oracle.c`` (FP64, Neumaier-compensated, threaded).
* :class:`ReferenceEngine` - the reference's own CPU engine
  (``NewMultiDimensionalScaling``) compiled from its sources into
  ``oracle/_ref/libmdsref.so`` where the reference tree is available.
"""
from .oracle import (  # noqa: F401
    ReferenceEngine,
    build,
    evaluate,
    gradient,
    log_likelihood,
    port_eval_rows,
    port_eval_rows_f32,
    reference_available,
    reference_root,
    sum_of_increments,
    sweep_rows,
)
