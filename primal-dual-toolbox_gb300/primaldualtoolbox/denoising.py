"""primaldualtoolbox.denoising -- TV and TGV^2 denoising (python/pyDenoising.cpp:39-94)."""
from __future__ import annotations

import numpy as np

from . import _lib
from ._core import TgvParameters, TvParameters, _Optimizer

__all__ = ["TgvParameters", "TvParameters", "TgvOptimizer_2f", "TvOptimizer_2f", "TgvOptimizer_2c",
           "TvOptimizer_2c"]


class TvOptimizer_2f(_Optimizer):
    """ROF: min_u TV(u) + Lambda/2 ||u - f||^2 for a real float32 image (tvoptimizer.cu:76-125)."""
    _kind = _lib.OPT_TV
    _dtype = np.float32
    _params_cls = TvParameters
    _tgv = False
    _with_op = False


class TgvOptimizer_2f(_Optimizer):
    """TGV^2-L2 denoising of a real float32 image (tgvoptimizer.cu:80-141)."""
    _kind = _lib.OPT_TGV
    _dtype = np.float32
    _params_cls = TgvParameters
    _with_op = False


class TvOptimizer_2c(TvOptimizer_2f):
    _dtype = np.complex64


class TgvOptimizer_2c(TgvOptimizer_2f):
    _dtype = np.complex64
