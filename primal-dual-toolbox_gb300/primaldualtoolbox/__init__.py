"""primaldualtoolbox -- GB300-native primal-dual TV / TGV^2 engine with the reference toolbox's Python API.

    import primaldualtoolbox
    op = primaldualtoolbox.mri.MriCartesianRemoveROOSOperator()
    op.setCoilSens(sens); op.setMask(mask)
    opt = primaldualtoolbox.mri.TgvMriOptimizer_2c3c()
    opt.getParameters().max_iter = 1000
    opt.setOperator(op); opt.setNoisyData(rawdata); opt.solve(); u = opt.getResult()

Everything runs in libpdt.so (hand-written CUDA for sm_103a); there is no CPU fallback.
"""
from . import batch, denoising, mri  # noqa: F401
from ._lib import LIB_PATH, PdtError, launch_count, pinned_empty  # noqa: F401

__version__ = "0.1.0"
