"""SliceStream (overlapped upload / solve / download with reused operators) against solving each slice
on its own, and in-place constant replacement."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _solo(pdt, case, max_iter):
    op = pdt.mri.MriCartesianRemoveROOSOperator()
    op.setCoilSens(case["sens"])
    op.setMask(case["mask"])
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.alpha1, prm.alpha0, prm.reduction, prm.max_iter = 0.05, 0.1, 0.5, max_iter
    opt.setOperator(op)
    opt.setNoisyData(case["rawdata"])
    opt.solve()
    return opt.getResult()


def test_slice_stream_equals_individual_solves(pdt):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox import pipeline, synthetic

    cases = [synthetic.cartesian_case(C=4, H=64, W=48, roos=True, seed=s) for s in range(5)]
    cases[3]["mask"] = cases[0]["mask"]  # repeated masks and a changed one in between
    cases[4]["mask"] = cases[0]["mask"]
    stream = pipeline.SliceStream(C=4, H=64, W=48, roos=True, alpha1=0.05, alpha0=0.1, reduction=0.5, max_iter=60,
                                  torch=torch)
    got = list(stream.run(cases))
    assert [i for i, _ in got] == list(range(5))
    for (i, img), case in zip(got, cases):
        assert rel_l2(img, _solo(pdt, case, 60)) <= 1e-6, i


def test_replace_constant_matches_fresh_operator(pdt):
    from primaldualtoolbox import synthetic

    a = synthetic.cartesian_case(C=3, H=64, W=48, roos=False, seed=11)
    b = synthetic.cartesian_case(C=3, H=64, W=48, roos=False, seed=12)
    op = pdt.mri.MriCartesianOperator()
    op.setCoilSens(a["sens"])
    op.setMask(a["mask"])
    first = op.adjoint(a["rawdata"])
    op.replaceCoilSens(b["sens"])
    op.replaceMask(b["mask"])
    fresh = pdt.mri.MriCartesianOperator()
    fresh.setCoilSens(b["sens"])
    fresh.setMask(b["mask"])
    assert np.array_equal(op.adjoint(b["rawdata"]), fresh.adjoint(b["rawdata"]))
    assert not np.array_equal(first, fresh.adjoint(a["rawdata"]))
    with pytest.raises(pdt.PdtError):
        op.replaceConstant(2, b["mask"])  # no third constant
    with pytest.raises(pdt.PdtError):
        op.replaceConstant(0, b["mask"][None].astype(np.complex64)[0])  # rank 2 for a rank-3 constant
