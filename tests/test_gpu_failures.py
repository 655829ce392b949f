"""Failure detection on the device, without a GPU fault.

* Non-finite values: the with-operator solvers check every new u and v for NaN / Inf inside the primal
  kernel and raise PDT_ERR_NUMERIC at the next synchronous call. The reference has no such check (its
  solve loop only checks kernel launches, tgvmrioptimizer.cu:163-198). The failure is made on the host:
  noisy data with a NaN or an Inf on a sampled phase-encode line.
* Bounded waits: every mbarrier wait of the tensor-core kernels gives up after 200 ms, records an error
  word, drains its own copies and MMAs and frees its tensor memory; the next synchronous call raises
  PDT_ERR_TIMEOUT. pdt_debug_drop_arrival makes the kernels withhold one arrival (a barrier phase that
  nothing completes), so the wait runs out; afterwards the same operator, solver and network must give
  correct results again, which shows that the context stayed usable.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

PDT_ERR_NUMERIC = 8
PDT_ERR_TIMEOUT = 9


def _case(C=4, H=64, W=48, seed=1):
    from primaldualtoolbox import synthetic

    return synthetic.cartesian_case(C=C, H=H, W=W, roos=True, seed=seed)


def _solver(pdt, case, f, max_iter=30):
    op = pdt.mri.MriCartesianRemoveROOSOperator()
    op.setCoilSens(case["sens"])
    op.setMask(case["mask"])
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.max_iter, prm.alpha1, prm.alpha0, prm.reduction = max_iter, case["alpha1"], case["alpha0"], 0.5
    opt.setOperator(op)
    opt.setNoisyData(f)
    return op, opt


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_non_finite_data_raises_numeric(pdt, oracle, bad):
    case = _case()
    f = case["rawdata"].copy()
    col = int(np.nonzero((case["mask"] != 0).any(axis=0))[0][3])  # a sampled phase-encode line
    f[1, 10, col] = bad
    _, opt = _solver(pdt, case, f)
    with pytest.raises(pdt.PdtError) as ei:
        opt.solve()
    assert ei.value.status == PDT_ERR_NUMERIC
    assert "Non-finite" in str(ei.value)
    # the flag was cleared: clean data on the same optimizer solves and matches the oracle
    opt.setNoisyData(case["rawdata"])
    opt.setInput0(np.zeros((32, 48), np.complex64))
    opt.solve()
    ref = oracle.op_solve("cartesian_roos", case["sens"], case["mask"], case["rawdata"], "tgv_mri",
                          alpha0=case["alpha0"], alpha1=case["alpha1"], reduction=0.5, max_iter=30,
                          u0=np.zeros((32, 48), np.complex64), prec=32)
    assert rel_l2(opt.getResult(), ref) <= 1e-4


def test_non_finite_on_unsampled_line_is_harmless(pdt):
    """Data on lines the mask never samples never reaches u (the reference masks it before every adjoint)."""
    case = _case(seed=2)
    f = case["rawdata"].copy()
    col = int(np.nonzero(~(case["mask"] != 0).any(axis=0))[0][0])
    f[0, 5, col] = np.nan
    _, opt = _solver(pdt, case, f)
    opt.solve()
    assert np.isfinite(opt.getResult()).all()


def test_non_finite_checked_on_a_stream(pdt):
    torch = pytest.importorskip("torch")
    case = _case(seed=3)
    f = case["rawdata"].copy()
    col = int(np.nonzero((case["mask"] != 0).any(axis=0))[0][0])
    f[2, 0, col] = np.nan
    _, opt = _solver(pdt, case, torch.from_numpy(f).cuda())
    s = torch.cuda.Stream()
    opt.solve(stream=s)  # asynchronous: no check yet
    with pytest.raises(pdt.PdtError) as ei:
        opt.checkFinite(stream=s)
    assert ei.value.status == PDT_ERR_NUMERIC
    opt.checkFinite(stream=s)  # cleared


@pytest.fixture
def tensor_rows():
    old = os.environ.get("PDT_CARTESIAN_TUNE")
    os.environ["PDT_CARTESIAN_TUNE"] = "2,2,2,1,0,1,1,4,4"
    yield
    if old is None:
        os.environ.pop("PDT_CARTESIAN_TUNE", None)
    else:
        os.environ["PDT_CARTESIAN_TUNE"] = old


def _drop(pdt, on):
    from primaldualtoolbox import _lib

    _lib.check(_lib.lib.pdt_debug_drop_arrival(ctypes.c_int(1 if on else 0)))


@pytest.mark.parametrize("C,H,W", [(3, 64, 48), (15, 640, 368)])
def test_tensor_row_wait_gives_up_and_recovers(pdt, oracle, tensor_rows, C, H, W):
    case = _case(C=C, H=H, W=W, seed=4)
    op, opt = _solver(pdt, case, case["rawdata"], max_iter=1)  # each give-up costs a 200 ms wait
    tuning = op.tuning()  # prepares (and pins) the tensor-core rows before the hook is armed
    assert "rows_fwd=tensor_dft" in tuning and "rows_adj=tensor_dft" in tuning, tuning
    k = case["rawdata"]
    want = oracle.op_apply("cartesian_roos", case["sens"], case["mask"], k, adjoint=True)
    _drop(pdt, True)
    try:
        with pytest.raises(pdt.PdtError) as ei:
            op.adjoint(k)
        assert ei.value.status == PDT_ERR_TIMEOUT and "gave up a bounded wait" in str(ei.value)
        with pytest.raises(pdt.PdtError) as ei:
            opt.solve()
        assert ei.value.status == PDT_ERR_TIMEOUT
    finally:
        _drop(pdt, False)
    # same operator and context afterwards: correct again
    assert rel_l2(op.adjoint(k), want) <= 1e-5
    op2, opt2 = _solver(pdt, case, case["rawdata"], max_iter=25)
    opt2.solve()
    ref = oracle.op_solve("cartesian_roos", case["sens"], case["mask"], case["rawdata"], "tgv_mri",
                          alpha0=case["alpha0"], alpha1=case["alpha1"], reduction=0.5, max_iter=25, prec=32)
    assert rel_l2(opt2.getResult(), ref) <= 1e-4


def test_convolution_wait_gives_up_and_recovers(pdt):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox import warmstart

    net = warmstart.WarmStartNet(seed=5)
    rng = np.random.default_rng(5)
    u0 = torch.from_numpy((rng.standard_normal((1, 48, 64)) + 1j * rng.standard_normal((1, 48, 64)))
                          .astype(np.complex64)).cuda()
    ua = torch.empty_like(u0)
    va = torch.empty((1, 2, 48, 64), dtype=torch.complex64, device="cuda")
    net.predict(u0, ua, va)
    want_u, want_v = ua.cpu().numpy(), va.cpu().numpy()
    _drop(pdt, True)
    try:
        with pytest.raises(pdt.PdtError) as ei:
            net.predict(u0, ua, va)
        assert ei.value.status == PDT_ERR_TIMEOUT
    finally:
        _drop(pdt, False)
    net.predict(u0, ua, va)
    assert np.array_equal(ua.cpu().numpy(), want_u) and np.array_equal(va.cpu().numpy(), want_v)
