"""Edge cases of the Cartesian TGV-MRI path against the oracle: no sampled phase-encode line at all, a
single coil, max_iter = 0 (one iteration), a fully sampled mask, and a generic (non-split) FFT length."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _solve(pdt, kind, sens, mask, f, max_iter, alpha1=0.05, reduction=0.5):
    op = (pdt.mri.MriCartesianRemoveROOSOperator if kind == "cartesian_roos" else pdt.mri.MriCartesianOperator)()
    op.setCoilSens(sens)
    op.setMask(mask)
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.max_iter, prm.alpha1, prm.alpha0, prm.reduction = max_iter, alpha1, 2 * alpha1, reduction
    opt.setOperator(op)
    opt.setNoisyData(f)
    opt.solve()
    return opt.getResult()


def _ref(oracle, kind, sens, mask, f, max_iter, alpha1=0.05, reduction=0.5):
    return oracle.op_solve(kind, sens, mask, f, "tgv_mri", alpha0=float(np.float32(2 * alpha1)),
                           alpha1=float(np.float32(alpha1)), reduction=float(np.float32(reduction)),
                           max_iter=max_iter, prec=32)


def test_mask_without_sampled_lines(pdt, oracle):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=3, H=64, W=48, roos=True, seed=21)
    mask = np.zeros_like(case["mask"])
    got = _solve(pdt, "cartesian_roos", case["sens"], mask, case["rawdata"], 30)
    ref = _ref(oracle, "cartesian_roos", case["sens"], mask, case["rawdata"], 30)
    assert np.all(np.isfinite(got)) and np.abs(got).max() == 0 and np.abs(ref).max() == 0


@pytest.mark.parametrize("C,H,W,roos,max_iter", [(1, 64, 48, False, 40), (1, 128, 96, True, 40),
                                                 (4, 64, 48, True, 0), (2, 50, 30, False, 40)])
def test_small_edge_solves(pdt, oracle, C, H, W, roos, max_iter):
    from primaldualtoolbox import synthetic

    kind = "cartesian_roos" if roos else "cartesian"
    case = synthetic.cartesian_case(C=C, H=H, W=W, roos=roos, seed=C + H + W)
    got = _solve(pdt, kind, case["sens"], case["mask"], case["rawdata"], max_iter)
    ref = _ref(oracle, kind, case["sens"], case["mask"], case["rawdata"], max_iter)
    assert rel_l2(got, ref) <= 1e-4


def test_fully_sampled_mask(pdt, oracle):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=3, H=64, W=64, roos=False, seed=22)
    mask = np.ones_like(case["mask"])
    got = _solve(pdt, "cartesian", case["sens"], mask, case["rawdata"], 40)
    ref = _ref(oracle, "cartesian", case["sens"], mask, case["rawdata"], 40)
    assert rel_l2(got, ref) <= 1e-4
