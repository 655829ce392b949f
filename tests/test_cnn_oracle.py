"""The oracle's restatement of the warm-start network: its backward pass against finite differences
(BF16 rounding off), so that it can serve as the checker of the GPU gradients."""
import numpy as np


def _params(seed, n_layers_scale=2.0):
    rng = np.random.default_rng(seed)
    sizes = [(9 * 32 * 2, 9 * 2), (32, 0)] + [(9 * 32 * 32, 9 * 32), (32, 0)] * 6 + [(9 * 8 * 32, 9 * 32), (8, 0)]
    parts = []
    for n, fan in sizes:
        parts.append(rng.standard_normal(n) * (np.sqrt(2.0 / fan) * 0.5 if fan else 0.05))
    return np.concatenate(parts).astype(np.float32)


def test_cnn_oracle_gradient_finite_differences(oracle):
    rng = np.random.default_rng(0)
    B, H, W = 1, 6, 7
    c = lambda *s: (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)
    u0, ut, vt = c(B, H, W), c(B, H, W), c(B, 2, H, W)
    p = _params(1)
    loss, g = oracle.cnn_grad_exact(p, u0, ut, vt)
    # probe a few parameters of every layer (weights and biases)
    offsets = np.cumsum([0, 576, 32] + [9216, 32] * 6 + [2304, 8])
    picks = []
    for k in range(len(offsets) - 1):
        lo, hi = offsets[k], offsets[k + 1]
        picks += list(rng.integers(lo, hi, size=2))
    for i in picks:
        h = 1e-4 * max(1.0, abs(float(p[i])))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        hp = float(pp[i]) - float(pm[i])
        fd = (oracle.cnn_grad_exact(pp, u0, ut, vt)[0] - oracle.cnn_grad_exact(pm, u0, ut, vt)[0]) / hp
        assert abs(fd - g[i]) <= 2e-3 * max(1.0, abs(g[i])) + 1e-6, (i, fd, g[i])
