"""GPU parity of the radial operators (MriRadialOperator / MriRadialSinglecoilOperator).

The reference computes these with gpuNUFFT, which is not shipped with it, so results parity with the
reference is unpinned; the engine is checked against the oracle's FP64 restatement of the same
Kaiser-Bessel gridding NUFFT (rel-L2 <= 1e-5), against the exact non-uniform DFT (the approximation error
the kernel width allows), for adjointness (<= 1e-5), and in the TGV-MRI solver against the FP32-mirror
oracle (rel-L2 <= 1e-4).
"""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def radial_traj(n_spokes, n_ro, golden=False):
    """(2, Ns) float32 trajectory: row 0 = imag(k), row 1 = real(k) as in bin/mri_radial_test.py."""
    if golden:
        ang = np.arange(n_spokes) * np.pi * (np.sqrt(5) - 1) / 2
    else:
        ang = np.arange(n_spokes) * np.pi / n_spokes
    r = (np.arange(n_ro) - n_ro / 2) / n_ro
    k = (r[:, None] * np.exp(1j * ang[None, :])).ravel()
    return np.array([k.imag, k.real]).astype(np.float32), k


def _op(pdt, N, osf, kw, traj, dcf, sens):
    cfg = {"osf": osf, "sector_width": 8, "kernel_width": kw, "img_dim": N}
    if sens is None:
        op = pdt.mri.MriRadialSinglecoilOperator(cfg)
        op.setTrajectory(traj)
        op.setDcf(dcf)
    else:
        op = pdt.mri.MriRadialOperator(cfg)
        op.setTrajectory(traj)
        op.setDcf(dcf)
        op.setCoilSens(sens)
    return op


def _rand_c(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("N,osf,kw,C", [(32, 1.5, 3, 3), (32, 2.0, 5, 2), (48, 2.0, 3, 1), (64, 1.5, 3, 0)])
def test_radial_operator_matches_oracle(pdt, oracle, N, osf, kw, C):
    rng = np.random.default_rng(N + C)
    traj, k = radial_traj(24, 2 * N, golden=True)
    dcf = (np.sqrt(np.abs(k)) + 0.05).astype(np.float32)[None, :]
    sens = _rand_c(rng, (C, N, N)) if C else None
    op = _op(pdt, N, osf, kw, traj, dcf, sens)
    u = _rand_c(rng, (N, N))
    y = _rand_c(rng, (max(C, 1), traj.shape[1]))
    fwd, adj = op.forward(u), op.adjoint(y)
    assert fwd.shape == (max(C, 1), traj.shape[1]) and adj.shape == (N, N)
    assert rel_l2(fwd, oracle.radial_apply(traj, dcf, sens, u, N, osf, kw, "forward")) <= 1e-5
    assert rel_l2(adj, oracle.radial_apply(traj, dcf, sens, y, N, osf, kw, "adjoint")) <= 1e-5
    lhs, rhs = np.vdot(y, fwd), np.vdot(adj, u)
    assert abs(lhs - rhs) / (np.linalg.norm(fwd) * np.linalg.norm(y)) <= 1e-5


def test_radial_nufft_accuracy_vs_ndft(pdt, oracle):
    rng = np.random.default_rng(1)
    N = 32
    traj, k = radial_traj(16, 64)
    dcf = np.ones((1, traj.shape[1]), dtype=np.float32)
    sens = _rand_c(rng, (2, N, N))
    u = _rand_c(rng, (N, N))
    exact = oracle.radial_apply(traj, dcf, sens, u, N, 2.0, 5, "ndft")
    assert rel_l2(_op(pdt, N, 2.0, 5, traj, dcf, sens).forward(u), exact) <= 2e-4
    assert rel_l2(_op(pdt, N, 1.5, 3, traj, dcf, sens).forward(u), exact) <= 3e-2


def test_radial_brain_trajectory_fixture(pdt, oracle):
    """data/brain_trajectory.npy: 512 readout samples x 64 uniform spokes, prepared as in bin/mri_radial_test.py
    (k_col = [imag(k), real(k)], dcf = sqrt|k|), 256 x 256 image, 4 coils, osf 2, kernel width 3."""
    k = np.load(os.path.join(GOLDEN, "brain_trajectory.npy")).ravel()
    traj = np.array([k.imag, k.real]).astype(np.float32)
    dcf = np.sqrt(np.abs(k)).astype(np.float32)[None, :]
    rng = np.random.default_rng(2)
    N = 256
    sens = _rand_c(rng, (4, N, N))
    op = _op(pdt, N, 2, 3, traj, dcf, sens)
    u = _rand_c(rng, (N, N))
    y = _rand_c(rng, (4, traj.shape[1]))
    assert rel_l2(op.forward(u), oracle.radial_apply(traj, dcf, sens, u, N, 2.0, 3, "forward")) <= 1e-5
    assert rel_l2(op.adjoint(y), oracle.radial_apply(traj, dcf, sens, y, N, 2.0, 3, "adjoint")) <= 1e-5


@pytest.mark.parametrize("multi", [True, False])
def test_radial_tgv_mri_solve(pdt, oracle, multi):
    rng = np.random.default_rng(3)
    N = 32
    traj, k = radial_traj(20, 64, golden=True)
    dcf = np.sqrt(np.abs(k)).astype(np.float32)[None, :]
    sens = None
    if multi:
        from primaldualtoolbox import synthetic

        sens = synthetic.coil_maps(4, N, N, seed=3)
    truth = synthetic_phantom(N)
    op = _op(pdt, N, 2, 3, traj, dcf, sens)
    f = op.forward(truth) + 0.01 * _rand_c(rng, (4 if multi else 1, traj.shape[1]))
    opt = pdt.mri.TgvMriOptimizer_2c2c()
    prm = opt.getParameters()
    prm.max_iter, prm.alpha1, prm.alpha0, prm.reduction = 200, 0.02, 0.04, 0.1
    opt.setOperator(op)
    opt.setNoisyData(f)
    opt.solve()
    ref = oracle.radial_solve(traj, dcf, sens, f, N, 2.0, 3, "tgv_mri", alpha0=0.04, alpha1=0.02, reduction=0.1,
                              max_iter=200, prec=32)
    assert rel_l2(opt.getResult(), ref) <= 1e-4


def synthetic_phantom(N):
    from primaldualtoolbox import synthetic

    return synthetic.mri_phantom(N, N, seed=0)


def test_radial_config5_slice_200_iterations(pdt, oracle):
    """One full radial slice of the benchmark: 256 x 256, 12 coils, 64 golden-angle spokes x 512 samples,
    Kaiser-Bessel width 3 on a 1.5x grid, density weights sqrt|k|, 200 TGV-MRI iterations (reduction 2^-8)
    against the FP32-mirror oracle (about 20 s on 16 host cores)."""
    from primaldualtoolbox import synthetic

    N, C = 256, 12
    traj, k = radial_traj(64, 512, golden=True)
    dcf = np.sqrt(np.abs(k)).astype(np.float32)[None, :]
    sens = synthetic.coil_maps(C, N, N, seed=0)
    op = _op(pdt, N, 1.5, 3, traj, dcf, sens)
    f = op.forward(synthetic.mri_phantom(N, N, seed=0))
    rng = np.random.default_rng(0)
    f = f + (0.01 * np.abs(f).max() * (rng.standard_normal(f.shape) + 1j * rng.standard_normal(f.shape))).astype(
        np.complex64)
    a1 = float(np.float32(0.02 * float(np.abs(op.adjoint(f)).max())))
    opt = pdt.mri.TgvMriOptimizer_2c2c()
    prm = opt.getParameters()
    prm.max_iter, prm.alpha1, prm.alpha0, prm.reduction = 199, a1, 2 * a1, 2.0 ** -8
    opt.setOperator(op)
    opt.setNoisyData(f)
    opt.solve()
    ref = oracle.radial_solve(traj, dcf, sens, f, N, 1.5, 3, "tgv_mri", alpha0=2 * a1, alpha1=a1,
                              reduction=2.0 ** -8, max_iter=199, prec=32)
    assert rel_l2(opt.getResult(), ref) <= 1e-4
