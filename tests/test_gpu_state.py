"""Full solver-state export and import (getState / setState over pdt_opt_get_field / pdt_opt_set_field).

The reference keeps u, u-bar, v, v-bar, p, q and the k-space dual r in TgvMriOptimizer's members
(tgvmrioptimizer.h:121-140) and resets v, p, q (setInput0, tgvmrioptimizer.cu:62-79) and r (setNoisyData,
:81-91) whenever a solve is set up, so a solve cannot be resumed in another optimizer there. Here every
field can be read and written: importing an exported state into a fresh optimizer and solving must give
bitwise what the original optimizer gives when it simply continues.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cart(pdt, case, roos, kind="tgv_mri", lam=1.0):
    op = (pdt.mri.MriCartesianRemoveROOSOperator if roos else pdt.mri.MriCartesianOperator)()
    op.setCoilSens(case["sens"])
    op.setMask(case["mask"])
    cls = {"tgv_mri": pdt.mri.TgvMriOptimizer_2c3c, "tgv_op": pdt.mri.TgvOptimizer_2c3c,
           "tv_op": pdt.mri.TvOptimizerWithOp_2c3c}[kind]
    opt = cls()
    prm = opt.getParameters()
    if kind != "tv_op":
        prm.alpha1, prm.alpha0 = case["alpha1"], case["alpha0"]
    if kind != "tgv_mri":
        prm.Lambda = lam
    opt.setOperator(op)
    opt.setNoisyData(case["rawdata"])
    return opt, prm


@pytest.mark.parametrize("kind,roos,shape", [("tgv_mri", True, (4, 64, 48)), ("tgv_mri", True, (15, 640, 368)),
                                             ("tgv_op", False, (3, 32, 24)), ("tv_op", False, (3, 32, 24))])
def test_state_import_resumes_bitwise(pdt, kind, roos, shape):
    from primaldualtoolbox import synthetic

    C, H, W = shape
    case = synthetic.cartesian_case(C=C, H=H, W=W, roos=roos, seed=4)
    a, pa = _cart(pdt, case, roos, kind)
    pa.max_iter = 42  # 43 iterations: two graph replays and an odd remainder, so parity flips
    a.solve()
    state = a.getState()
    assert ("r" in state) and ("qxy" in state) == (kind != "tv_op")
    assert state["r"].shape == case["rawdata"].shape
    # r is held on the sampled phase-encode lines only; it reads back as 0 on the others
    unsampled = ~(case["mask"] != 0).any(axis=0)
    assert np.all(state["r"][:, :, unsampled] == 0)
    assert np.any(state["r"] != 0)

    b, pb = _cart(pdt, case, roos, kind)
    b.setInput0UV(np.zeros_like(state["u"]))  # sizes the state (TgvOptimizerWithOp has no setInput0)
    b.setState(state)
    back = b.getState()
    for k in state:
        assert np.array_equal(back[k], state[k]), k
    pa.max_iter = pb.max_iter = 30
    a.solve()
    b.solve()
    assert np.array_equal(a.getResult(), b.getResult())
    for k in ("px", "py", "r"):
        assert np.array_equal(a.getField(k), b.getField(k)), k


def test_state_import_on_device_arrays(pdt):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=3, H=64, W=48, roos=True, seed=8)
    a, pa = _cart(pdt, case, True)
    pa.max_iter = 20
    a.solve()
    host = a.getState()
    dev = {k: torch.from_numpy(v).cuda() for k, v in host.items()}
    b, pb = _cart(pdt, case, True)
    b.setInput0(dev["u"])
    b.setState(dev)
    out = torch.empty_like(dev["r"])
    b.getField("r", out=out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), host["r"])
    pa.max_iter = pb.max_iter = 10
    a.solve()
    b.solve()
    assert np.array_equal(a.getResult(), b.getResult())


def test_state_denoising_and_radial(pdt):
    from primaldualtoolbox import synthetic

    f = synthetic.tv_phantom(64, 80, seed=2)[0].astype(np.float32)
    a = pdt.denoising.TgvOptimizer_2f()
    a.setNoisyData(f)
    a.getParameters().max_iter = 17
    a.solve()
    st = a.getState()
    assert "r" not in st
    b = pdt.denoising.TgvOptimizer_2f()
    b.setNoisyData(f)
    b.setInput0UV(f)
    b.setState(st)
    a.getParameters().max_iter = b.getParameters().max_iter = 9
    a.solve()
    b.solve()
    assert np.array_equal(a.getResult(), b.getResult())

    N = 32
    ang = np.arange(16) * np.pi * (np.sqrt(5) - 1) / 2
    r = (np.arange(64) - 32) / 64
    k = (r[:, None] * np.exp(1j * ang[None, :])).ravel()
    traj = np.array([k.imag, k.real]).astype(np.float32)
    dcf = np.sqrt(np.abs(k)).astype(np.float32)[None, :]
    sens = synthetic.coil_maps(3, N, N, seed=1)

    def radial_opt():
        op = pdt.mri.MriRadialOperator({"osf": 1.5, "sector_width": 8, "kernel_width": 3, "img_dim": N})
        op.setTrajectory(traj)
        op.setDcf(dcf)
        op.setCoilSens(sens)
        opt = pdt.mri.TgvMriOptimizer_2c2c()
        prm = opt.getParameters()
        prm.alpha1, prm.alpha0 = 0.02, 0.04
        opt.setOperator(op)
        return op, opt, prm

    op, ra, pra = radial_opt()
    fr = op.forward(synthetic.mri_phantom(N, N, seed=1))
    ra.setNoisyData(fr)
    pra.max_iter = 25
    ra.solve()
    st = ra.getState()
    assert st["r"].shape == fr.shape
    _, rb, prb = radial_opt()
    rb.setNoisyData(fr)
    rb.setInput0(st["u"])
    rb.setState(st)
    pra.max_iter = prb.max_iter = 12
    ra.solve()
    rb.solve()
    assert np.array_equal(ra.getResult(), rb.getResult())


def test_state_errors(pdt):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=2, H=32, W=32, roos=False, seed=0)
    opt, _ = _cart(pdt, case, False)
    with pytest.raises(pdt.PdtError, match="no result yet|no state yet"):
        opt.setField("px", np.zeros((32, 32), np.complex64))
    opt.setInput0(np.zeros((32, 32), np.complex64))
    with pytest.raises(pdt.PdtError, match="no dual state yet"):
        opt.getField("r")  # setNoisyData reset r and no solve has run since
    with pytest.raises(ValueError, match="shape"):
        opt.setField("r", np.zeros((2, 32, 31), np.complex64))
