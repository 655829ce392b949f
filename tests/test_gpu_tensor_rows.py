"""Tensor-core DFT row passes (tcgen05, TF32 hi/lo split) forced on, against the oracle.

PDT_CARTESIAN_TUNE pins the launch configuration of operators prepared while it is set; its fields 6 and 7
select the tensor-core forward and adjoint rows (where the operator supports them: even W, and for the
adjoint a lane-FFT column length). Tolerances as in test_gpu_parity: operators rel-L2 <= 1e-5 against the
FP64 oracle, solvers <= 1e-4 against the FP32-mirror oracle.
"""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

SHAPES = [(15, 640, 368, True), (3, 64, 48, True), (2, 32, 16, False), (1, 64, 368, False), (4, 128, 96, False),
          (5, 320, 320, True)]


@pytest.fixture
def tensor_rows():
    old = os.environ.get("PDT_CARTESIAN_TUNE")
    os.environ["PDT_CARTESIAN_TUNE"] = "2,2,2,1,0,1,1,4,4"
    yield
    if old is None:
        os.environ.pop("PDT_CARTESIAN_TUNE", None)
    else:
        os.environ["PDT_CARTESIAN_TUNE"] = old


@pytest.mark.parametrize("C,H,W,roos", SHAPES)
def test_tensor_rows_match_oracle(pdt, oracle, tensor_rows, C, H, W, roos):
    rng = np.random.default_rng(C * 7 + H + W)
    sens = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
    mask = np.zeros((H, W), dtype=np.float32)
    mask[:, rng.random(W) < 0.3] = 1
    mask[:, W // 2] = 1
    kind = "cartesian_roos" if roos else "cartesian"
    op = pdt.mri.MriCartesianRemoveROOSOperator() if roos else pdt.mri.MriCartesianOperator()
    op.setCoilSens(sens)
    op.setMask(mask)
    Hi = H // 2 if roos else H
    u = (rng.standard_normal((Hi, W)) + 1j * rng.standard_normal((Hi, W))).astype(np.complex64)
    assert rel_l2(op.forward(u), oracle.op_apply(kind, sens, mask, u)) <= 1e-5
    tuning = op.tuning()
    assert "rows_fwd=tensor_dft" in tuning and "rows_adj=tensor_dft" in tuning, tuning
    f = oracle.op_apply(kind, sens, mask, u).astype(np.complex64)
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.max_iter, prm.alpha1, prm.alpha0, prm.reduction = 40, 0.01, 0.02, 0.5
    opt.setOperator(op)
    opt.setNoisyData(f)
    opt.solve()
    ref = oracle.op_solve(kind, sens, mask, f, alpha0=0.02, alpha1=0.01, reduction=0.5, max_iter=40, prec=32)
    assert rel_l2(opt.getResult(), ref) <= 1e-4
    op.tuning()  # raises if a bounded wait in a tensor-core kernel gave up


def test_dual_in_adjoint_launch_matches_own_kernel(pdt, oracle, monkeypatch):
    """The solvers' dual update, run in the SMs the tensor-core adjoint rows leave free (extra blocks of that
    launch), gives the iterates of the dual kernel on its own forked stream (same per-pixel arithmetic)."""
    C, H, W = 15, 640, 368
    rng = np.random.default_rng(11)
    sens = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
    mask = np.zeros((H, W), dtype=np.float32)
    mask[:, rng.random(W) < 0.3] = 1
    mask[:, W // 2] = 1
    u = (rng.standard_normal((H // 2, W)) + 1j * rng.standard_normal((H // 2, W))).astype(np.complex64)
    f = oracle.op_apply("cartesian_roos", sens, mask, u).astype(np.complex64)
    monkeypatch.setenv("PDT_CARTESIAN_TUNE", "8,2,2,8,0,0,1,3,3")  # 3 x 40 row tiles: 32 SMs free

    def solve(tgv):
        op = pdt.mri.MriCartesianRemoveROOSOperator()
        op.setCoilSens(sens)
        op.setMask(mask)
        tuning = op.tuning()
        opt = pdt.mri.TgvMriOptimizer_2c3c() if tgv else pdt.mri.TvOptimizerWithOp_2c3c()
        prm = opt.getParameters()
        prm.max_iter = 30
        if tgv:
            prm.alpha1, prm.alpha0, prm.reduction = 0.01, 0.02, 0.5
        opt.setOperator(op)
        opt.setNoisyData(f)
        opt.solve()
        op.tuning()  # raises if a bounded wait in a tensor-core kernel gave up
        return opt.getResult(), tuning

    for tgv in (True, False):
        monkeypatch.delenv("PDT_NO_FUSED_DUAL", raising=False)
        fused, tuning = solve(tgv)
        assert "solver_dual=adjoint_launch(30_blocks)" in tuning, tuning
        monkeypatch.setenv("PDT_NO_FUSED_DUAL", "1")
        forked, tuning = solve(tgv)
        assert "solver_dual" not in tuning, tuning
        assert rel_l2(fused, forked) <= 1e-6
