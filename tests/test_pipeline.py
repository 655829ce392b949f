"""Data-layout converters of primaldualtoolbox.pipeline (the reference scripts' Python and MATLAB layouts)."""
import numpy as np
import pytest


def _rand_c(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def test_cartesian_matlab_layout():
    from primaldualtoolbox import pipeline

    rng = np.random.default_rng(0)
    raw = _rand_c(rng, (4, 16, 12))  # Python (C, FE, PE)
    sens = _rand_c(rng, (4, 16, 12))
    mask = (rng.random((16, 12)) < 0.5).astype(np.float64)
    m = pipeline.cartesian_from_matlab(np.transpose(raw, (1, 2, 0)), np.transpose(sens, (1, 2, 0)), mask)
    assert np.array_equal(m["rawdata"], raw) and np.array_equal(m["sens"], sens)
    assert m["mask"].dtype == np.float32 and np.array_equal(m["mask"], mask.astype(np.float32))
    assert m["rawdata"].flags.c_contiguous


def test_roos_crop_rows():
    from primaldualtoolbox import pipeline

    img = np.arange(640)[:, None] * np.ones((1, 3))
    c = pipeline.roos_crop(img)
    assert c.shape == (320, 3) and c[0, 0] == 161 and c[-1, 0] == 480


def test_radial_layouts_agree():
    from primaldualtoolbox import pipeline

    rng = np.random.default_rng(1)
    nfe, nsp, C = 8, 5, 3
    k = (rng.random((nfe, nsp)) - 0.5 + 1j * (rng.random((nfe, nsp)) - 0.5)).astype(np.complex64)
    raw_py = _rand_c(rng, (C, nfe, nsp))
    py = pipeline.radial_inputs(k, raw_py)
    assert py["trajectory"].shape == (2, nfe * nsp) and py["rawdata"].shape == (C, nfe * nsp)
    assert np.array_equal(py["trajectory"][0], np.imag(k).ravel()) and np.array_equal(py["trajectory"][1],
                                                                                       np.real(k).ravel())
    assert np.allclose(py["dcf"][0], np.sqrt(np.abs(k.ravel())))
    # the same acquisition in MATLAB layout: samples enumerate in column order, so match them by trajectory
    raw_m = np.transpose(raw_py, (1, 2, 0))  # (FE, spokes, C)
    m = pipeline.radial_inputs(k, raw_m, layout="matlab")
    order_py = {complex(t0, t1): i for i, (t0, t1) in enumerate(py["trajectory"].T)}
    perm = [order_py[complex(t0, t1)] for t0, t1 in m["trajectory"].T]
    assert np.array_equal(m["rawdata"], py["rawdata"][:, perm])
    mo = pipeline.radial_inputs(k, raw_m, layout="matlab", trajectory_order="matlab")
    assert np.array_equal(mo["trajectory"], m["trajectory"][::-1])


def test_load_array_npy_and_mat(tmp_path):
    from primaldualtoolbox import pipeline

    scipy_io = pytest.importorskip("scipy.io")
    a = np.arange(12, dtype=np.float32).reshape(3, 4)
    np.save(tmp_path / "a.npy", a)
    scipy_io.savemat(tmp_path / "a.mat", {"mask": a})
    assert np.array_equal(pipeline.load_array(str(tmp_path / "a.npy")), a)
    assert np.array_equal(pipeline.load_array(str(tmp_path / "a.mat")), a)
    scipy_io.savemat(tmp_path / "b.mat", {"x": a, "y": a})
    with pytest.raises(ValueError):
        pipeline.load_array(str(tmp_path / "b.mat"))
    assert np.array_equal(pipeline.load_array(str(tmp_path / "b.mat"), name="y"), a)
