"""FP64 metrics on the GPU (energy, operator norm, distances) and the (u, v) warm start, against the oracle."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _setup(pdt, C=4, H=64, W=48, seed=1, max_iter=60, reduction=1.0):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=C, H=H, W=W, roos=True, seed=seed)
    op = pdt.mri.MriCartesianRemoveROOSOperator()
    op.setCoilSens(case["sens"])
    op.setMask(case["mask"])
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.max_iter, prm.alpha1, prm.alpha0, prm.reduction = max_iter, case["alpha1"], case["alpha0"], reduction
    opt.setOperator(op)
    opt.setNoisyData(case["rawdata"])
    return op, opt, case


def test_energy_matches_oracle(pdt, oracle):
    op, opt, case = _setup(pdt)
    opt.solve()
    e = opt.energy()
    u, vx, vy = opt.getField("u"), opt.getField("vx"), opt.getField("vy")
    ref = oracle.tgv_energy("cartesian_roos", case["sens"], case["mask"], case["rawdata"], u, vx, vy,
                            float(np.float32(case["alpha0"])), float(np.float32(case["alpha1"])))
    assert abs(e["total"] - ref) / ref <= 1e-5
    assert e["data"] > 0 and e["first_order"] > 0 and e["second_order"] >= 0


def test_energy_decreases_over_the_run(pdt, oracle):
    # primal-dual iterates need not lower the primal energy at every step (the duals start at zero);
    # over long spans they approach the minimum from above, like the FP64 oracle's
    op, opt, case = _setup(pdt, max_iter=0)
    opt.setInput0(op.adjoint(case["rawdata"]))
    e = {0: opt.energy()["total"]}
    done = 0
    for n in (2000, 8000):
        opt.getParameters().max_iter = n - done - 1
        opt.solve()
        done = n
        e[n] = opt.energy()["total"]
    assert e[8000] < e[2000] < e[0]


def test_operator_norm_is_one_for_normalised_coils(pdt):
    # sum_c |c|^2 = 1 and at least one fully sampled line: ||K|| = 1 (the TGV step sizes assume <= 1)
    op, _, _ = _setup(pdt)
    n = op.norm(iters=60)
    assert abs(n - 1.0) < 2e-3


def test_warm_start_uv_and_fields(pdt):
    op, opt, case = _setup(pdt, max_iter=0)
    rng = np.random.default_rng(0)
    u0 = (rng.standard_normal((32, 48)) + 1j * rng.standard_normal((32, 48))).astype(np.complex64)
    v0 = (rng.standard_normal((2, 32, 48)) + 1j * rng.standard_normal((2, 32, 48))).astype(np.complex64)
    opt.setInput0UV(u0, v0)
    assert np.array_equal(opt.getField("u"), u0)
    assert np.array_equal(opt.getField("vx"), v0[0])
    assert np.array_equal(opt.getField("vbary"), v0[1])
    assert not np.any(opt.getField("qxy"))


def test_dist2(pdt):
    torch = pytest.importorskip("torch")
    a = torch.randn(1000, dtype=torch.complex64, device="cuda")
    b = torch.randn(1000, dtype=torch.complex64, device="cuda")
    got = pdt.dist2(a, b)
    want = float((a.cpu().numpy().astype(np.complex128) - b.cpu().numpy()).__abs__().__pow__(2).sum())
    assert abs(got - want) / want < 1e-12


@pytest.mark.parametrize("variant,lam", [("tgv_mri", 1.0), ("tgv_op", 2.0), ("tv_op", 0.5)])
def test_gap_matches_oracle(pdt, oracle, variant, lam):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=4, H=64, W=48, roos=False, seed=3)
    op = pdt.mri.MriCartesianOperator()
    op.setCoilSens(case["sens"])
    op.setMask(case["mask"])
    cls = {"tgv_mri": pdt.mri.TgvMriOptimizer_2c3c, "tgv_op": pdt.mri.TgvOptimizer_2c3c,
           "tv_op": pdt.mri.TvOptimizerWithOp_2c3c}[variant]
    opt = cls()
    prm = opt.getParameters()
    prm.max_iter = 79
    if variant == "tgv_mri":
        prm.reduction = 1.0
    else:
        prm.Lambda = lam
    a0, a1 = (float(np.float32(case["alpha0"])), float(np.float32(case["alpha1"])))
    if variant != "tv_op":
        prm.alpha0, prm.alpha1 = a0, a1
    opt.setOperator(op)
    opt.setNoisyData(case["rawdata"])
    opt.solve()
    got = opt.gap()
    _, st = oracle.op_solve("cartesian", case["sens"], case["mask"], case["rawdata"], variant, alpha0=a0, alpha1=a1,
                            reduction=1.0, lam=lam, max_iter=79, prec=32, return_state=True)
    ref = oracle.op_gap("cartesian", case["sens"], case["mask"], case["rawdata"], st, variant, alpha0=a0, alpha1=a1,
                        lam=lam)
    for k in ("primal", "dual", "norm_khr"):
        assert abs(got[k] - ref[k]) <= 1e-5 * abs(ref[k]), k
    for k in ("gap", "residual_u") + (() if variant == "tv_op" else ("residual_v",)):
        assert abs(got[k] - ref[k]) <= 2e-3 * abs(ref[k]), k
    assert got["gap"] > 0
