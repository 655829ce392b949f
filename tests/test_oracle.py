"""CPU checks of the oracle (the checker the GPU parity tests rely on).

Pins: the reference's adjointness test (tests/main_adjointness_test.cu:28-64: double2, coil sens
{10,10,5}, {0,1} mask, PASSED below 1e-12), numpy.fft for the orthonormal FFT ImageUtilities provides,
the reference's mask fixtures, and internal consistency (FP32 mirror vs FP64).
"""
import os

import numpy as np
import pytest

from conftest import rel_l2

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 10, 23, 46, 97, 192, 320, 368, 384, 640])
def test_fft_matches_numpy(oracle, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert np.abs(oracle.fft1d(x) - np.fft.fft(x)).max() <= 1e-12 * max(1, n)
    assert np.abs(oracle.fft1d(x, inverse=True) - np.fft.ifft(x) * n).max() <= 1e-12 * max(1, n)


def _ref_adjointness_inputs(kind, seed=42):
    rng = np.random.default_rng(seed)
    sens = rng.random((5, 10, 10)) + 1j * rng.random((5, 10, 10))
    mask = rng.integers(0, 2, (10, 10)).astype(np.float64)
    Hi = 5 if kind == "cartesian_roos" else 10
    u = rng.random((Hi, 10)) + 1j * rng.random((Hi, 10))
    pshape = (10, 10) if kind == "sampling" else (5, 10, 10)
    p = rng.random(pshape) + 1j * rng.random(pshape)
    return sens, mask, u, p


@pytest.mark.parametrize("kind", ["cartesian", "cartesian_roos", "sampling"])
def test_reference_adjointness_test(oracle, kind):
    """tests/main_adjointness_test.cu: |<Au,p> - <u,A^H p>| < 1e-12 per component in double."""
    sens, mask, u, p = _ref_adjointness_inputs(kind)
    Au = oracle.op_apply(kind, sens, mask, u, prec=64)
    Atp = oracle.op_apply(kind, sens, mask, p, adjoint=True, prec=64)
    lhs = np.sum(Au * np.conj(p))
    rhs = np.sum(u * np.conj(Atp))
    assert abs(lhs.real - rhs.real) < 1e-12 and abs(lhs.imag - rhs.imag) < 1e-12


@pytest.mark.parametrize("shape", [(4, 16, 12), (3, 10, 10), (2, 64, 48)])
@pytest.mark.parametrize("roos", [False, True])
def test_cartesian_matches_numpy_model(oracle, shape, roos):
    """Even sizes: the reference's ifftshift / fftshift2 pair equals numpy's, so the operator is
    mask . fftshift(fft2(ifftshift(sens . pad(u)), norm=ortho))."""
    from primaldualtoolbox import synthetic

    C, H, W = shape
    rng = np.random.default_rng(1)
    sens = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    mask = (rng.random((H, W)) > 0.5).astype(np.float64)
    Hi = H // 2 if roos else H
    u = rng.standard_normal((Hi, W)) + 1j * rng.standard_normal((Hi, W))
    k = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    kind = "cartesian_roos" if roos else "cartesian"
    assert np.abs(oracle.op_apply(kind, sens, mask, u) - synthetic.cartesian_forward(u, sens, mask, roos)).max() < 1e-12
    assert np.abs(oracle.op_apply(kind, sens, mask, k, adjoint=True)
                  - synthetic.cartesian_adjoint(k, sens, mask, roos)).max() < 1e-12


def test_roos_offset_matches_reference_formula():
    from primaldualtoolbox import synthetic

    # mricartesianoperator.cu:341: unsigned int FE_idx = size[1] * 0.25f + 1
    assert synthetic.roos_offset(640) == 161
    assert synthetic.roos_offset(768) == 193
    assert synthetic.roos_offset(10) == 3


def test_odd_size_shift_conventions(oracle):
    """For odd sizes the reference's ifftshift uses mid = int((n+1)/2) (a roll by ceil(n/2))."""
    C, H, W = 1, 7, 5
    sens = np.ones((C, H, W), dtype=np.complex128)
    mask = np.ones((H, W))
    u = np.zeros((H, W), dtype=np.complex128)
    u[0, 0] = 1.0
    k = oracle.op_apply("cartesian", sens, mask, u)
    # input at (0,0) lands at FFT slot (4, 3): the spectrum is a pure phase ramp of unit modulus / sqrt(N)
    assert np.allclose(np.abs(k[0]), 1 / np.sqrt(H * W))


def test_fp32_mirror_tracks_fp64(oracle):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=3, H=32, W=24, roos=True, seed=4)
    args = ("cartesian_roos", case["sens"], case["mask"], case["rawdata"], "tgv_mri")
    kw = dict(alpha0=case["alpha0"], alpha1=case["alpha1"], reduction=1.0, max_iter=300)
    u32 = oracle.op_solve(*args, prec=32, **kw)
    u64 = oracle.op_solve(*args, prec=64, **kw)
    assert rel_l2(u32, u64) < 1e-4


def test_tgv_energy_decreases(oracle):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=3, H=32, W=24, roos=True, seed=5)
    args = ("cartesian_roos", case["sens"], case["mask"], case["rawdata"], "tgv_mri")
    kw = dict(alpha0=case["alpha0"], alpha1=case["alpha1"], reduction=1.0, prec=64)
    energies = []
    for it in (0, 50, 400):
        u, st = oracle.op_solve(*args, max_iter=it, return_state=True, **kw)
        energies.append(oracle.tgv_energy("cartesian_roos", case["sens"], case["mask"], case["rawdata"],
                                          st["u"], st["vx"], st["vy"], case["alpha0"], case["alpha1"]))
    assert energies[0] > energies[1] > energies[2]


def test_alpha_schedule(oracle):
    # tgvmrioptimizer.cu:150-155: geometric interpolation from alpha to alpha*reduction over max_iter
    a0, a1 = oracle.alpha_schedule(2.0, 1.0, 1e-2, 100, 0)
    assert a0 == pytest.approx(2.0, rel=1e-6) and a1 == pytest.approx(1.0, rel=1e-6)
    a0, a1 = oracle.alpha_schedule(2.0, 1.0, 1e-2, 100, 100)
    assert a0 == pytest.approx(0.02, rel=1e-5) and a1 == pytest.approx(0.01, rel=1e-5)
    a0, a1 = oracle.alpha_schedule(2.0, 1.0, 1e-2, 100, 50)
    assert a0 == pytest.approx(0.2, rel=1e-5)


def test_tv_denoise_fp32_vs_fp64(oracle):
    rng = np.random.default_rng(0)
    f = rng.random((40, 30)).astype(np.float32)
    u32 = oracle.tv_solve(f, lam=10, max_iter=200, prec=32)
    u64 = oracle.tv_solve(f.astype(np.float64), lam=10, max_iter=200, prec=64)
    assert rel_l2(u32, u64) < 1e-5


def test_reference_masks_are_line_masks(oracle):
    """data/mask_cartesian_{random4,regular4}.npy: 117 / 96 sampled lines of 384, 28 centre lines."""
    rnd = np.load(os.path.join(GOLDEN, "mask_random4_lines.npy"))
    reg = np.load(os.path.join(GOLDEN, "mask_regular4_lines.npy"))
    assert len(rnd) == 117
    assert set(range(178, 206)) <= set(rnd.tolist())
    assert 90 <= len(reg) <= 130
    # the oracle's adjointness on the reference's own mask (single coil, 768 x 384)
    m = np.zeros((768, 384))
    m[:, rnd] = 1
    rng = np.random.default_rng(0)
    u = rng.standard_normal((768, 384)) + 1j * rng.standard_normal((768, 384))
    p = rng.standard_normal((768, 384)) + 1j * rng.standard_normal((768, 384))
    Au = oracle.op_apply("sampling", None, m, u)
    Atp = oracle.op_apply("sampling", None, m, p, adjoint=True)
    assert abs(np.vdot(p, Au) - np.vdot(Atp, u)) / (np.linalg.norm(Au) * np.linalg.norm(p)) < 1e-12


def test_op_solve_continues_from_state(oracle):
    # at reduction 1 two solves of 10 and 20 iterations are the 30-iteration solve (up to the rounding of
    # exp(log alpha) in the schedule, which depends on max_iter)
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=2, H=32, W=24, roos=True, seed=7)
    args = ("cartesian_roos", case["sens"], case["mask"], case["rawdata"], "tgv_mri")
    kw = dict(alpha0=case["alpha0"], alpha1=case["alpha1"], reduction=1.0, prec=64)
    _, st = oracle.op_solve(*args, max_iter=9, return_state=True, **kw)
    u2 = oracle.op_solve(*args, max_iter=19, state=st, **kw)
    u = oracle.op_solve(*args, max_iter=29, **kw)
    assert rel_l2(u2, u) < 1e-12
    assert rel_l2(oracle.op_solve(*args, max_iter=19, **kw), u) > 1e-3  # the state did carry over


@pytest.mark.parametrize("variant,lam", [("tgv_mri", 1.0), ("tgv_op", 2.0), ("tv_op", 0.5)])
def test_primal_dual_gap_closes(oracle, variant, lam):
    from primaldualtoolbox import synthetic

    case = synthetic.cartesian_case(C=3, H=32, W=24, roos=False, seed=8)
    kw = dict(alpha0=case["alpha0"], alpha1=case["alpha1"], lam=lam)
    gaps = []
    for it in (30, 300, 3000):
        _, st = oracle.op_solve("cartesian", case["sens"], case["mask"], case["rawdata"], variant, reduction=1.0,
                                max_iter=it - 1, prec=64, return_state=True, **kw)
        gaps.append(oracle.op_gap("cartesian", case["sens"], case["mask"], case["rawdata"], st, variant, **kw))
    assert gaps[0]["gap"] > gaps[1]["gap"] > gaps[2]["gap"] > -1e-9 * gaps[2]["primal"]
    assert gaps[2]["residual_u"] < 0.05 * gaps[0]["residual_u"]
    if variant != "tv_op":
        assert gaps[2]["residual_v"] < 0.05 * gaps[0]["residual_v"]
