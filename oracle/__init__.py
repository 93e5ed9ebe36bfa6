"""CPU oracle for the lbmminiapp collide-stream path (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference arm may import this package, and only as the checker or the timed
CPU baseline.  The product package ``lbmminiapp_gb300`` never imports it.

* :mod:`oracle.core` -- ctypes wrapper of ``lbm_oracle.c`` (C restatement of
  the reference algorithm, OpenMP) plus numpy helpers (lattice tables, raw
  slot <-> logical population conversion, macroscopic readouts).
* :mod:`oracle.ref`  -- ctypes wrapper of the reference's own CPU kernels
  compiled by ``build_ref.sh`` (only where the reference sources exist).
"""
