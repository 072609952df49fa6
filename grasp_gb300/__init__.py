"""grasp_gb300 - GRASP's relativistic CI hot path (R^k / I(ab) tables, SETHAM,
Davidson) as hand-written sm_103a CUDA behind a C ABI (include/grasp_gpu.h).

Layout:
  csrc/       CUDA kernels and the C ABI (libgraspgpu.so)
  core.py     Context / HMatrix: the reference-named host interface
  formats.py  GRASP file formats (Fortran unformatted records)
  build.py    nvcc build recipe (sm_103a)
"""
from .core import FP64, SPLIT, Context, HMatrix, maneig_batched  # noqa: F401
from ._lib import GGError  # noqa: F401

__all__ = ["Context", "HMatrix", "GGError", "FP64", "SPLIT", "maneig_batched"]
