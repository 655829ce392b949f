"""The cuFFT companion's launch chain, run by torch.fft on the CPU, against the FP64 oracle: it restates the
reference's shift, scaling, ROOS and combine conventions (so the GPU comparison beside cuFFT is meaningful)."""
import numpy as np
import pytest

from conftest import rel_l2


@pytest.mark.parametrize("C,H,W,roos", [(3, 16, 12, False), (2, 30, 7, True), (4, 64, 48, True), (1, 9, 5, False)])
def test_companion_matches_oracle(oracle, C, H, W, roos):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox.cufft_companion import CartesianCufft

    rng = np.random.default_rng(C + H + W)
    sens = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
    mask = (rng.random((H, W)) < 0.5).astype(np.float32)
    Hi = H // 2 if roos else H
    u = (rng.standard_normal((Hi, W)) + 1j * rng.standard_normal((Hi, W))).astype(np.complex64)
    k = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
    comp = CartesianCufft(torch.from_numpy(sens), torch.from_numpy(mask), roos, torch)
    kind = "cartesian_roos" if roos else "cartesian"
    assert rel_l2(comp.forward(torch.from_numpy(u)).numpy(), oracle.op_apply(kind, sens, mask, u)) <= 1e-5
    assert rel_l2(comp.adjoint(torch.from_numpy(k)).numpy(),
                  oracle.op_apply(kind, sens, mask, k, adjoint=True)) <= 1e-5
