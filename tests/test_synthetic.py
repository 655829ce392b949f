"""Seeded synthetic inputs with the shapes and statistics the benchmark configurations name."""
import numpy as np

from primaldualtoolbox import synthetic


def test_tv_phantom():
    f, clean = synthetic.tv_phantom(128, 96, seed=3)
    assert f.shape == (128, 96) and f.dtype == np.float32
    assert 0.08 < np.std(f - clean) < 0.12
    f2, _ = synthetic.tv_phantom(128, 96, seed=3)
    assert np.array_equal(f, f2)


def test_coil_maps_normalised():
    s = synthetic.coil_maps(15, 64, 48, seed=0)
    assert s.shape == (15, 64, 48) and s.dtype == np.complex64
    assert np.allclose(np.sum(np.abs(s) ** 2, axis=0), 1.0, atol=1e-5)


def test_line_mask():
    m = synthetic.line_mask(640, 368, accel=4, center=28, seed=0)
    cols = np.nonzero(m.any(axis=0))[0]
    assert len(cols) == 92
    assert set(range(170, 198)) <= set(cols.tolist())
    assert np.array_equal(m, np.repeat(m[:1], 640, axis=0))
    r = synthetic.line_mask(640, 368, accel=4, center=28, seed=0, kind="regular")
    assert r.any(axis=0).sum() >= 92


def test_cartesian_case():
    c = synthetic.cartesian_case(C=4, H=64, W=48, roos=True, seed=0)
    assert c["rawdata"].shape == (4, 64, 48) and c["truth"].shape == (32, 48)
    assert np.all(c["rawdata"][:, :, c["mask"][0] == 0] == 0)
    assert c["alpha0"] == 2 * c["alpha1"] > 0
