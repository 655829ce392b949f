"""The warm-start network: the engine's tensor-core forward / backward kernels against the oracle's FP64
restatement (BF16 rounding at the same storage points), training, and the energy fallback rule."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _batch(rng, B, H, W):
    c = lambda *s: (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)
    u0 = c(B, H, W)
    ut = u0 + 0.3 * c(B, H, W)
    vt = 0.2 * c(B, 2, H, W)
    return u0, ut, vt


def _layer_slices(net):
    sizes = [9 * 32 * 2, 32] + [9 * 32 * 32, 32] * 6 + [9 * 8 * 32, 8]
    out, o = [], 0
    for n in sizes:
        out.append(slice(o, o + n))
        o += n
    assert o == net.num_params
    return out


def test_cnn_gradients_match_oracle(pdt, oracle):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox.warmstart import WarmStartNet

    rng = np.random.default_rng(0)
    B, H, W = 2, 24, 40
    u0, ut, vt = _batch(rng, B, H, W)
    net = WarmStartNet(seed=3)
    # larger residual branches than the default initialisation, so every layer carries gradient
    p = net.get_params()
    net.set_params(p * 2.0)
    p = net.get_params()
    loss = net.train_step(torch.from_numpy(u0).cuda(), torch.from_numpy(ut).cuda(), torch.from_numpy(vt).cuda(),
                          lr=0.0)
    g = net.grads()
    ref_loss, ref_g, _ = oracle.cnn_grad(p, u0, ut, vt)
    assert abs(loss - ref_loss) / ref_loss <= 1e-3
    for sl in _layer_slices(net):
        if np.linalg.norm(ref_g[sl]) > 0:
            assert rel_l2(g[sl], ref_g[sl]) <= 2e-2


def test_cnn_forward_matches_oracle(pdt, oracle):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox.warmstart import WarmStartNet

    rng = np.random.default_rng(1)
    B, H, W = 2, 20, 33
    u0, ut, vt = _batch(rng, B, H, W)
    net = WarmStartNet(seed=4)
    net.set_params(net.get_params() * 2.0)
    u = torch.empty((B, H, W), dtype=torch.complex64, device="cuda")
    v = torch.empty((B, 2, H, W), dtype=torch.complex64, device="cuda")
    net.predict(torch.from_numpy(u0).cuda(), u, v)
    _, _, out8 = oracle.cnn_grad(net.get_params(), u0, ut, vt)
    s = np.abs(u0).reshape(B, -1).max(axis=1)[:, None, None]
    u_ref = u0 + s * (out8[..., 0] + 1j * out8[..., 1])
    v_ref = np.stack([s * (out8[..., 2] + 1j * out8[..., 3]), s * (out8[..., 4] + 1j * out8[..., 5])], axis=1)
    assert rel_l2(u.cpu().numpy() - u0, u_ref - u0) <= 1e-2
    assert rel_l2(v.cpu().numpy(), v_ref) <= 1e-2


def test_cnn_training_reduces_loss(pdt):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox.warmstart import WarmStartNet

    rng = np.random.default_rng(2)
    u0, ut, vt = _batch(rng, 4, 32, 48)
    # a learnable target: smoothed versions of the input
    ut = (u0 + np.roll(u0, 1, axis=1) + np.roll(u0, 1, axis=2)) / 3
    vt = np.stack([np.roll(u0, 1, axis=2) - u0, np.roll(u0, 1, axis=1) - u0], axis=1) * 0.5
    d = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (u0, ut, vt)]
    net = WarmStartNet(seed=5)
    first = net.train_step(*d, lr=0.0)
    for _ in range(150):
        last = net.train_step(*d, lr=2e-3)
    assert last < 0.5 * first


def test_warm_start_keeps_the_lower_energy(pdt):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox import synthetic
    from primaldualtoolbox.warmstart import WarmStartNet, warm_start

    case = synthetic.cartesian_case(C=4, H=64, W=48, roos=True, seed=7)
    op = pdt.mri.MriCartesianRemoveROOSOperator()
    op.setCoilSens(case["sens"])
    op.setMask(case["mask"])
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.alpha1, prm.alpha0, prm.max_iter = case["alpha1"], case["alpha0"], 10
    opt.setOperator(op)
    f = torch.from_numpy(case["rawdata"]).cuda()
    opt.setNoisyData(f)
    u0 = torch.empty((32, 48), dtype=torch.complex64, device="cuda")
    op.adjoint(f, out=u0)
    for scale in (1.0, 40.0):  # an untrained net, and one made deliberately bad
        net = WarmStartNet(seed=9)
        net.set_params(net.get_params() * scale)
        info = warm_start(opt, net, u0, torch)
        assert opt.energy()["total"] == pytest.approx(min(info["energy_network"], info["energy_plain"]), rel=1e-9)
    assert info["used"] == "plain"
