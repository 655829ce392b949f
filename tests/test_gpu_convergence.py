"""Time to rel-L2 1e-4 of the fixed-alpha TGV-MRI iteration: the reference's step sizes versus the
dual-weighted ones (warmstart.DUAL_WEIGHTED_STEPS), and the learned warm start on a held-out case.

Both step-size choices are the same primal-dual iteration with tau sigma |K|^2 < 1, so they converge to
the same saddle point; the dual-weighted one gets there many times sooner because the slow tail of the
reference's iteration is the convergence of the duals p, q (sigma / tau = 2 there, 1024 here).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver(pdt, case, f, roos):
    op = (pdt.mri.MriCartesianRemoveROOSOperator if roos else pdt.mri.MriCartesianOperator)()
    op.setCoilSens(case["sens"])
    op.setMask(case["mask"])
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.reduction, prm.alpha1 = 1.0, case["alpha1"]
    prm.alpha0 = 2 * prm.alpha1
    opt.setOperator(op)
    opt.setNoisyData(f)
    return op, opt, prm


def _iterations_to(opt, prm, u_star, chunk, cap, target=1e-4):
    prm.max_iter = chunk - 1
    it = 0
    while it < cap:
        opt.solve()
        it += chunk
        e = np.linalg.norm(opt.getResult() - u_star) / np.linalg.norm(u_star)
        if e <= target:
            return it, e
    return None, e


def _u_star(pdt, case, roos, steps, iters, reference_check=False):
    """The dual-weighted iterate after `iters` iterations; with reference_check, also the relative change
    of u over 2000 further iterations of the same optimizer (all state kept) with the reference's steps."""
    _, o, p = _solver(pdt, case, case["rawdata"], roos)
    o.setSteps(*steps)
    p.max_iter = iters - 1
    o.solve()
    u = o.getResult()
    if not reference_check:
        return u
    o.setSteps(0, 0)
    p.max_iter = 1999
    o.solve()
    return u, float(np.linalg.norm(o.getResult() - u) / np.linalg.norm(u))


def test_dual_weighted_steps_same_solution_sooner(pdt):
    from primaldualtoolbox import synthetic, warmstart

    case = synthetic.cartesian_case(C=4, H=96, W=64, roos=False, seed=21)
    steps = warmstart.DUAL_WEIGHTED_STEPS
    u_star, change = _u_star(pdt, case, False, steps, 40000, reference_check=True)
    assert change <= 2e-5  # the dual-weighted limit is a fixed point of the reference's iteration too
    _, plain, pp = _solver(pdt, case, case["rawdata"], False)
    n_plain, e_plain = _iterations_to(plain, pp, u_star, 1000, 300000)
    _, dual, pd = _solver(pdt, case, case["rawdata"], False)
    dual.setSteps(*steps)
    n_dual, _ = _iterations_to(dual, pd, u_star, 250, 60000)
    assert n_dual is not None
    assert n_plain is None or n_dual * 3 <= n_plain, (n_dual, n_plain, e_plain)


def test_learned_warm_start_on_held_out_case(pdt):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox import synthetic, warmstart

    if not os.path.exists(warmstart.CONFIG4_WEIGHTS):
        pytest.skip("no trained weights for the 15-coil 320 x 320 configuration")
    case = synthetic.cartesian_case(C=15, H=320, W=320, roos=False, accel=4, seed=900001)  # not a training seed
    steps = warmstart.DUAL_WEIGHTED_STEPS
    u_star = _u_star(pdt, case, False, steps, 40000)
    f = torch.from_numpy(case["rawdata"]).cuda()
    op, opt, prm = _solver(pdt, case, f, False)
    u0 = torch.empty((320, 320), dtype=torch.complex64, device="cuda")
    op.adjoint(f, out=u0)
    net = warmstart.WarmStartNet(weights=warmstart.CONFIG4_WEIGHTS)
    choice = warmstart.warm_start(opt, net, u0, torch)
    assert choice["used"] == "network", choice
    start = opt.getResult()
    d_net = np.linalg.norm(start - u_star) / np.linalg.norm(u_star)
    d_plain = np.linalg.norm(u0.cpu().numpy() - u_star) / np.linalg.norm(u_star)
    assert d_net < d_plain, (d_net, d_plain)
    opt.setSteps(*steps)
    n_warm, _ = _iterations_to(opt, prm, u_star, 250, 60000)
    _, plain, pp = _solver(pdt, case, f, False)
    plain.setInput0(u0)
    n_plain, e_plain = _iterations_to(plain, pp, u_star, 2000, 200000)
    assert n_warm is not None
    assert n_plain is None or n_warm < n_plain, (n_warm, n_plain, e_plain)


def test_dual_weighted_limit_is_a_fixed_point_of_the_fp64_oracle(pdt, oracle):
    """The state the GPU reaches with the dual-weighted steps, handed to the FP64 oracle of the reference
    iteration (reference steps, tgvmrioptimizer.cu:120-200) as its starting state: 3000 FP64 iterations
    move u by less than 1e-5 relative, so the limit is the reference method's converged solution."""
    from primaldualtoolbox import synthetic, warmstart

    case = synthetic.cartesian_case(C=3, H=48, W=32, roos=False, seed=31)
    _, o, p = _solver(pdt, case, case["rawdata"], False)
    o.setSteps(*warmstart.DUAL_WEIGHTED_STEPS)
    p.max_iter = 39999
    o.solve()
    st = o.getState()
    names = {"vbarx": "vbx", "vbary": "vby"}
    state = {names.get(k, k): v.astype(np.complex128) for k, v in st.items()}
    unsampled = ~(case["mask"] != 0).any(axis=0)
    # the engine does not hold r on never-sampled lines; the reference's r there is (r + sigma (0 - f)) / (1 + sigma)
    # iterated from 0, i.e. it tends to -f, which is 0 for these (masked) data
    assert np.all(case["rawdata"][:, :, unsampled] == 0)
    u64 = oracle.op_solve("cartesian", case["sens"], case["mask"], case["rawdata"], "tgv_mri",
                          alpha0=float(np.float32(case["alpha0"])), alpha1=float(np.float32(case["alpha1"])),
                          reduction=1.0, max_iter=2999, prec=64, state=state)
    assert np.linalg.norm(u64 - st["u"]) / np.linalg.norm(st["u"]) <= 1e-5
