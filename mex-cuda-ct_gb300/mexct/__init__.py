"""mexct: GB300 implementation of the mex-cuda-CT projection-operator path.

The compute lives in libmexct.so (CUDA, sm_103a) behind the C ABI of
``include/mexct.h``; this package is its Python mirror with the reference's MATLAB
function names (see :mod:`mexct.ops`).
"""
from . import _lib  # noqa: F401
from .ops import (  # noqa: F401
    CUDAmex_BP,
    CUDAmex_FP,
    CUDAmex_general3D_BP,
    CUDAmex_general3D_FP,
    CUDAmex_oscIter,
    CUDAmex_TVmin_3D,
    FBP_recon,
    general3D_BP_matched,
    parker_weight,
    preFilterSinogram,
)
from .solver import OSC_TV_recon  # noqa: F401
