"""primaldualtoolbox -- GB300-native primal-dual TV / TGV^2 engine with the reference toolbox's Python API.

    import primaldualtoolbox
    op = primaldualtoolbox.mri.MriCartesianRemoveROOSOperator()
    op.setCoilSens(sens); op.setMask(mask)
    opt = primaldualtoolbox.mri.TgvMriOptimizer_2c3c()
    opt.getParameters().max_iter = 1000
    opt.setOperator(op); opt.setNoisyData(rawdata); opt.solve(); u = opt.getResult()

Everything runs in libpdt.so (hand-written CUDA for sm_103a); there is no CPU fallback.
"""
from . import batch, denoising, mri, pipeline  # noqa: F401
from ._lib import LIB_PATH, PdtError, launch_count, pinned_empty  # noqa: F401


def dist2(a, b=None, stream=None):
    """sum |a - b|^2 of two device arrays (b optional), accumulated in FP64 on the GPU."""
    import ctypes

    import numpy as np

    from . import _lib

    dt = np.dtype(a.__cuda_array_interface__["typestr"])
    A = _lib.Buffer(a, dt)
    B = None if b is None else _lib.Buffer(b, dt)
    if not A.is_device or (B is not None and not B.is_device):
        raise TypeError("dist2 takes device arrays")
    n = int(np.prod(A.shape))
    out = ctypes.c_double()
    _lib.check(_lib.lib.pdt_dist2(_lib.C64 if dt == np.complex64 else _lib.F32, A.ptr, B.ptr if B else None, n,
                                  _lib.stream_handle(stream), ctypes.byref(out)))
    return out.value

__version__ = "0.1.0"
