"""GB300-native (sm_103a) collide-stream path of the lbmminiapp LBM proxy app.

The compute path is the CUDA library ``liblbm_gb300.so`` behind the C ABI of
``include/lbm_gb300.h``; this package is its host-side binding:

* :class:`Simulation` -- one library handle (geometry, state, time loop,
  readouts, kernel-level calls on caller buffers);
* :mod:`.reference_api` -- ``Parameters`` / ``PropagationAA`` /
  ``PropagationAB`` with the reference's method names, driven by the
  reference's input files;
* :mod:`.workloads` -- seeded synthetic inputs of the benchmark configs.
"""
from ._native import LBMError, lib, library_path  # noqa: F401
from .simulation import Simulation, cylinder  # noqa: F401

__all__ = ["Simulation", "cylinder", "LBMError", "lib", "library_path"]
