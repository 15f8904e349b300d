"""pyinla_gb300: the BTA solve at the centre of pyINLA, written for one NVIDIA GB300.

Public pieces:

* :mod:`pyinla_gb300.algs` -- drop-in for ``serinv.algs`` (``pobtaf, pobtas,
  pobtasi, pobtf, pobts, pobtsi``) used by the reference's ``SerinvSolver``;
* :class:`pyinla_gb300.solver.GB300SerinvSolver` -- drop-in for ``SerinvSolver``
  itself, with device-resident block buffers;
* the C ABI in ``include/pyinla_gb300.h`` (``libpyinla_gb300.so``), which the two
  above call through ctypes.

All arithmetic runs in the CUDA library; nothing falls back to the CPU.
"""
from ._lib import GBTAError, LIB_PATH, load

__all__ = ["GBTAError", "LIB_PATH", "load"]
__version__ = "0.1.0"
