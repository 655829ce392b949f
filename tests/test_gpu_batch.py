"""Batched solves: uneven problems (size, coils, acceleration, mask kind, optimizer, iteration count)
advanced together must give exactly what solving each alone gives (where the batch launches the same
kernels; widths with a separate forward-row split for concurrent launches, operators whose solo tuning
chose the tensor-core rows, which a batch replaces by the lane-FFT rows, and operators whose adjoint rows
run with fewer coil groups in a batch agree to FP32 rounding)."""
import re

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

CASES = [  # (C, H, W, roos, accel, mask kind, max_iter)
    (8, 192, 192, False, 2, "regular", 40),
    (12, 256, 256, False, 5, "random", 33),
    (5, 320, 320, True, 8, "random", 40),
    (15, 640, 368, True, 4, "random", 25),
    (3, 64, 48, True, 3, "regular", 40),
]


def _make(pdt, C, H, W, roos, accel, kind, max_iter, seed):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=C, H=H, W=W, roos=roos, accel=accel, mask_kind=kind, seed=seed)
    op = (pdt.mri.MriCartesianRemoveROOSOperator if roos else pdt.mri.MriCartesianOperator)()
    op.setCoilSens(case["sens"])
    op.setMask(case["mask"])
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.max_iter, prm.alpha1, prm.alpha0, prm.reduction = max_iter, case["alpha1"], case["alpha0"], 0.5
    opt.setOperator(op)
    opt.setNoisyData(case["rawdata"])
    opt.op_ref = op
    return opt, case


def test_batch_equals_individual_solves(pdt, oracle):
    solo, batched, cases = [], [], []
    for i, c in enumerate(CASES):
        o, case = _make(pdt, *c, seed=i)
        o.solve()
        solo.append(o.getResult())
        b, _ = _make(pdt, *c, seed=i)
        batched.append(b)
        cases.append(case)
    # a denoising problem rides along
    f = np.random.default_rng(9).random((100, 90)).astype(np.float32)
    den = pdt.denoising.TvOptimizer_2f()
    den.setNoisyData(f)
    den.getParameters().Lambda, den.getParameters().max_iter = 8.0, 57
    ref_den = pdt.denoising.TvOptimizer_2f()
    ref_den.setNoisyData(f)
    ref_den.getParameters().Lambda, ref_den.getParameters().max_iter = 8.0, 57
    ref_den.solve()
    bs = pdt.batch.BatchSolver(batched + [den])
    bs.solve()

    def same_kernels(tuning):
        """The batch launches what the solo solve launched: lane-FFT rows with the same coil groups."""
        if "tensor_dft" in tuning:
            return False
        solo_g = re.search(r"coil_groups=(\d+)", tuning)
        batch_g = re.search(r"batch_adj_groups=(\d+)", tuning)
        return solo_g is None or batch_g is None or solo_g.group(1) == batch_g.group(1)

    same = []
    for i, c in enumerate(CASES):
        o, _ = _make(pdt, *c, seed=i)
        same.append(same_kernels(o.op_ref.tuning()))
    for o, want, c, sk in zip(batched, solo, CASES, same):
        # batched rounds take the 23 x 16 forward-row split at width 368 (alone: 46 x 8), the lane-FFT rows
        # where the solo tuning chose the tensor-core rows, and at most two coil groups: FP32 rounding
        if c[2] == 368 or not sk:
            assert rel_l2(o.getResult(), want) <= 1e-5
        else:
            assert np.array_equal(o.getResult(), want)
    assert np.array_equal(den.getResult(), ref_den.getResult())
    # the small case and the 15 x 640 x 368 case against the oracle
    for i in (4, 3):
        c = CASES[i]
        ref = oracle.op_solve("cartesian_roos", cases[i]["sens"], cases[i]["mask"], cases[i]["rawdata"], "tgv_mri",
                              alpha0=cases[i]["alpha0"], alpha1=cases[i]["alpha1"], reduction=0.5, max_iter=c[6],
                              prec=32)
        assert rel_l2(batched[i].getResult(), ref) <= 1e-4, c
    # a second batched solve continues from the state, like a second solve() call
    bs.solve()
    for o in batched:
        assert np.isfinite(o.getResult()).all()


def test_batch_rejects_shared_operator(pdt):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=2, H=32, W=32, roos=False, seed=0)
    op = pdt.mri.MriCartesianOperator()
    op.setCoilSens(case["sens"])
    op.setMask(case["mask"])
    a, b = pdt.mri.TgvMriOptimizer_2c3c(), pdt.mri.TgvMriOptimizer_2c3c()
    a.setOperator(op)
    b.setOperator(op)
    bs = pdt.batch.BatchSolver([a])
    with pytest.raises(pdt.PdtError, match="distinct operators"):
        bs.add(b)
