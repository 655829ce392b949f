"""primaldualtoolbox.mri -- MRI operators and optimizers (python/pyMriReconstruction.cpp:112-268).

Array layouts as in the reference's Python samples (bin/mri_cartesian_test.py, bin/mri_radial_test.py):
Cartesian k-space and coil sensitivities ``(coils, FE, PE)`` complex64, masks ``(FE, PE)`` float32,
images ``(FE, PE)`` complex64 (``(FE/2, PE)`` for the readout-oversampling removal operator).
"""
from __future__ import annotations

import numpy as np

from . import _lib
from ._core import TgvMriParameters, TgvParameters, TvParameters, _Operator, _Optimizer

__all__ = ["TgvMriParameters", "TgvParameters", "TvParameters", "MriCartesianOperator",
           "MriCartesianRemoveROOSOperator", "MriRadialOperator", "MriRadialSinglecoilOperator",
           "MriSamplingOperator", "TgvMriOptimizer_2c3c", "TgvOptimizer_2c3c", "TvOptimizerWithOp_2c3c",
           "TgvMriOptimizer_2c2c", "TgvOptimizer_2c2c", "TvOptimizer_2c2c"]


class MriCartesianOperator(_Operator):
    """Multi-coil Cartesian operator: constants setCoilSens (#0) then setMask (#1), in that order.
    replaceCoilSens / replaceMask swap them in place for the next slice (no reference counterpart)."""
    _kind = _lib.OP_CARTESIAN
    _constant_types = ((np.complex64, _lib.C64), (np.float32, _lib.F32))

    def __init__(self):
        super().__init__(None)

    def setMask(self, mask):
        self._add_constant(mask, np.float32, _lib.F32)

    def setCoilSens(self, sens):
        self._add_constant(sens, np.complex64, _lib.C64)

    def replaceCoilSens(self, sens, stream=None):
        self.replaceConstant(0, sens, stream)

    def replaceMask(self, mask, stream=None):
        self.replaceConstant(1, mask, stream)


class MriCartesianRemoveROOSOperator(MriCartesianOperator):
    """Cartesian operator whose image is the central half of the readout (FE) field of view."""
    _kind = _lib.OP_CARTESIAN_ROOS


class MriSamplingOperator(_Operator):
    """Single-coil centred FFT + mask; constant setMask (#0)."""
    _kind = _lib.OP_SAMPLING
    _constant_types = ((np.float32, _lib.F32),)

    def __init__(self):
        super().__init__(None)

    def setMask(self, mask):
        self._add_constant(mask, np.float32, _lib.F32)

    def replaceMask(self, mask, stream=None):
        self.replaceConstant(0, mask, stream)


class MriRadialOperator(_Operator):
    """Radial multi-coil operator; config dict with osf, sector_width, kernel_width, img_dim.
    Constants in order: setTrajectory (2, Ns) float32, setDcf (1, Ns) float32, setCoilSens (C, N, N)."""
    _kind = _lib.OP_RADIAL
    _constant_types = ((np.float32, _lib.F32), (np.float32, _lib.F32), (np.complex64, _lib.C64))

    def __init__(self, config):
        super().__init__(config)

    def setTrajectory(self, traj):
        self._add_constant(traj, np.float32, _lib.F32)

    def setDcf(self, dcf):
        self._add_constant(dcf, np.float32, _lib.F32)

    def setCoilSens(self, sens):
        self._add_constant(sens, np.complex64, _lib.C64)

    def replaceTrajectory(self, traj, stream=None):
        self.replaceConstant(0, traj, stream)

    def replaceDcf(self, dcf, stream=None):
        self.replaceConstant(1, dcf, stream)

    def replaceCoilSens(self, sens, stream=None):
        self.replaceConstant(2, sens, stream)


class MriRadialSinglecoilOperator(_Operator):
    """Radial single-coil operator; constants setTrajectory then setDcf."""
    _kind = _lib.OP_RADIAL_SINGLECOIL
    _constant_types = ((np.float32, _lib.F32), (np.float32, _lib.F32))

    def __init__(self, config):
        super().__init__(config)

    def setTrajectory(self, traj):
        self._add_constant(traj, np.float32, _lib.F32)

    def setDcf(self, dcf):
        self._add_constant(dcf, np.float32, _lib.F32)

    def replaceTrajectory(self, traj, stream=None):
        self.replaceConstant(0, traj, stream)

    def replaceDcf(self, dcf, stream=None):
        self.replaceConstant(1, dcf, stream)


_OPS_3C = (MriCartesianOperator, MriCartesianRemoveROOSOperator)
_OPS_2C = (MriRadialOperator, MriRadialSinglecoilOperator, MriSamplingOperator)


class TgvMriOptimizer_2c3c(_Optimizer):
    """TGV^2 MRI reconstruction with alpha continuation for the Cartesian operators."""
    _kind = _lib.OPT_TGV_MRI
    _params_cls = TgvMriParameters
    _operators = _OPS_3C

    def setOperator(self, op):
        self._set_operator(op)

    def setInput0(self, u0, stream=None):
        self._set_input0(u0, stream)


class TgvOptimizer_2c3c(_Optimizer):
    """TGV^2 with an operator (TgvOptimizerWithOp), Cartesian operators."""
    _kind = _lib.OPT_TGV_OP
    _params_cls = TgvParameters
    _operators = _OPS_3C

    def setOperator(self, op):
        self._set_operator(op)


class TvOptimizerWithOp_2c3c(_Optimizer):
    """TV with an operator (TvOptimizerWithOp), Cartesian operators."""
    _kind = _lib.OPT_TV_OP
    _params_cls = TvParameters
    _tgv = False
    _operators = _OPS_3C

    def setOperator(self, op):
        self._set_operator(op)

    def setInput0(self, u0, stream=None):
        self._set_input0(u0, stream)


class TgvMriOptimizer_2c2c(TgvMriOptimizer_2c3c):
    """TGV^2 MRI reconstruction for the radial and sampling operators."""
    _operators = _OPS_2C


class TgvOptimizer_2c2c(TgvOptimizer_2c3c):
    _operators = _OPS_2C


class TvOptimizer_2c2c(_Optimizer):
    """TV with an operator (TvOptimizerWithOp), radial and sampling operators."""
    _kind = _lib.OPT_TV_OP
    _params_cls = TvParameters
    _tgv = False
    _operators = _OPS_2C

    def setOperator(self, op):
        self._set_operator(op)
