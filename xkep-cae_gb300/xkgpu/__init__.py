"""xkgpu: GB300 (sm_103a) assembly of the xkep-cae CR-beam + frictional-contact Newton iteration.

Hand-written CUDA kernels behind a C ABI (``include/xkgpu.h``), driven from
Python through ctypes on PyTorch-owned device memory.

* ``xkgpu.engine.AssemblyEngine``   device-resident per-increment detection and
  per-iteration assembly (the fast path)
* ``xkgpu.strategies``              drop-in replacements for the reference's
  Strategy-protocol objects and manager processes
* ``xkgpu.strand`` / ``xkgpu.workloads``  synthetic strand workloads
"""

from . import _lib  # noqa: F401

__all__ = ["_lib"]
__version__ = "0.1.0"
