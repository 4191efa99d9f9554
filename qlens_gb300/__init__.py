"""qlens_gb300 -- QLens's pixel-image likelihood on one GB300 (sm_103a).

The compute path is libqlpix.so (hand-written CUDA + C++ host runtime behind
the C ABI of include/qlpix.h).  ``PixelLikelihood`` mirrors the QLens calls a
fitting driver makes; see qlens_gb300/pixlike.py.
"""
from . import abi
from .abi import QLP_FP64, QLP_MIXED
from .pixlike import (PixelLikelihood, QLPixError, LibraryUnavailable, gaussian_psf, pixel_corners, load_library,
                      library_path)

__all__ = ["abi", "PixelLikelihood", "QLPixError", "LibraryUnavailable", "gaussian_psf", "pixel_corners",
           "load_library", "library_path", "QLP_FP64", "QLP_MIXED"]
