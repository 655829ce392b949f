"""The oracle pinned to the reference's own code.

tests/golden/ref_small.npz holds outputs of the reference's optimizer loops, TGV kernels and Cartesian
operators (src/optimizer/*, src/operator/mricartesianoperator.cu) compiled for the CPU by
oracle/ref_build.py against a host stand-in for ImageUtilities (tests/golden/make_ref_golden.py wrote
it). The oracle restatement (oracle/pdt_oracle.cpp) must reproduce them: the FP32 mirror the optimizers
(TV, TGV, TV / TGV with operator: bit for bit; TGV-MRI, whose FFTs round differently: rel-L2 <= 1e-6) and
the FP64 operators to rel-L2 <= 1e-6. Where the reference checkout is present, the library is built and
compared with the oracle on fresh inputs as well.
"""
import os

import numpy as np
import pytest

from conftest import rel_l2

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-6


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLDEN, "ref_small.npz"))


@pytest.mark.parametrize("key,kind", [("roos", "cartesian_roos"), ("cart", "cartesian")])
def test_operators_match_reference(oracle, gold, key, kind):
    s, m = gold[f"op_{key}_sens"], gold[f"op_{key}_mask"]
    assert rel_l2(oracle.op_apply(kind, s, m, gold[f"op_{key}_u"]), gold[f"op_{key}_fwd"]) <= TOL
    assert rel_l2(oracle.op_apply(kind, s, m, gold[f"op_{key}_k"], adjoint=True), gold[f"op_{key}_adj"]) <= TOL


@pytest.mark.parametrize("key,kind", [("tgvmri_roos", "cartesian_roos"), ("tgvmri_cart", "cartesian")])
def test_tgv_mri_matches_reference(oracle, gold, key, kind):
    a0, a1, red, it = gold[f"{key}_params"]
    u = oracle.op_solve(kind, gold[f"{key}_sens"], gold[f"{key}_mask"], gold[f"{key}_f"], "tgv_mri", alpha0=a0,
                        alpha1=a1, reduction=red, max_iter=int(it), prec=32)
    assert rel_l2(u, gold[f"{key}_u"]) <= TOL


def test_with_op_optimizers_match_reference_bitwise(oracle, gold):
    a0, a1 = gold["withop_alpha"]
    args = (gold["withop_sens"], gold["withop_mask"], gold["withop_f"])
    tgv = oracle.op_solve("cartesian", *args, "tgv_op", alpha0=a0, alpha1=a1, lam=2.0, max_iter=300, prec=32)
    tv = oracle.op_solve("cartesian", *args, "tv_op", lam=2.0, max_iter=300, prec=32)
    assert np.array_equal(tgv, gold["tgvop_u"])
    assert np.array_equal(tv, gold["tvop_u"])


def test_denoising_matches_reference_bitwise(oracle, gold):
    """TV-ROF on the 512 x 512 benchmark image for the stated 501 iterations, and TGV / complex TV."""
    assert np.array_equal(oracle.tv_solve(gold["rof_f"], lam=10.0, max_iter=500, prec=32), gold["rof_u"])
    assert np.array_equal(oracle.tgv_solve(gold["tgv_f"], lam=10.0, alpha0=0.2, alpha1=0.1, max_iter=200, prec=32),
                          gold["tgv_u"])
    assert np.array_equal(oracle.tgv_solve(gold["tgvc_f"], lam=10.0, alpha0=0.2, alpha1=0.1, max_iter=200,
                                           prec=32), gold["tgvc_u"])
    assert np.array_equal(oracle.tv_solve(gold["tgvc_f"], lam=10.0, max_iter=200, prec=32), gold["tvc_u"])


@pytest.fixture(scope="module")
def ref():
    from oracle import ref as r

    if not r.available():
        pytest.skip("the reference checkout is not present: oracle/_ref cannot be built here")
    return r


def test_reference_build_on_fresh_inputs(oracle, ref):
    """The reference compiled for the CPU against the oracle on inputs that no golden file holds."""
    from primaldualtoolbox import synthetic

    rng = np.random.default_rng(123)
    for roos, (C, H, W) in ((True, (2, 40, 30)), (False, (3, 24, 20))):
        kind = "cartesian_roos" if roos else "cartesian"
        c = synthetic.cartesian_case(C=C, H=H, W=W, roos=roos, seed=int(rng.integers(1000)))
        a1 = np.float32(c["alpha1"])
        want = ref.tgv_mri(roos, c["sens"], c["mask"], c["rawdata"], np.float32(2 * a1), a1, np.float32(0.05), 60)
        got = oracle.op_solve(kind, c["sens"], c["mask"], c["rawdata"], "tgv_mri", alpha0=float(2 * a1),
                              alpha1=float(a1), reduction=float(np.float32(0.05)), max_iter=60, prec=32)
        assert rel_l2(got, want) <= TOL
    f = rng.random((33, 27)).astype(np.float32)
    assert np.array_equal(oracle.tv_solve(f, lam=4.0, max_iter=50, prec=32), ref.denoise("tv", f, 4.0, 50))
