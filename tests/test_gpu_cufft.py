"""The hand-written fused FFT operators of libpdt.so checked beside cuFFT.

The companion (primaldualtoolbox.cufft_companion) runs the reference's own launch chain (shifts, batched
cuFFT fft2/ifft2 with orthonormal scaling, mask, conj-sens combine, ROOS pad/crop) through torch.fft on the
same device inputs. Both are FP32; tolerance rel-L2 <= 1e-5 for the operators and for one operator half of
a TGV-MRI iteration (k-space prox then adjoint).
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5

SHAPES = [(15, 640, 368, True), (4, 64, 48, False), (3, 320, 320, True), (2, 30, 7, False), (8, 256, 256, True)]


def _case(C, H, W, seed):
    rng = np.random.default_rng(seed)
    sens = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
    mask = np.zeros((H, W), dtype=np.float32)
    mask[:, rng.random(W) < 0.35] = 1
    return rng, sens, mask


@pytest.mark.parametrize("C,H,W,roos", SHAPES)
def test_operator_beside_cufft(pdt, C, H, W, roos):
    import torch

    from primaldualtoolbox.cufft_companion import CartesianCufft

    rng, sens, mask = _case(C, H, W, C * 100 + H + W)
    Hi = H // 2 if roos else H
    u = (rng.standard_normal((Hi, W)) + 1j * rng.standard_normal((Hi, W))).astype(np.complex64)
    k = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
    d = {n: torch.from_numpy(a).cuda() for n, a in (("sens", sens), ("mask", mask), ("u", u), ("k", k))}
    op = pdt.mri.MriCartesianRemoveROOSOperator() if roos else pdt.mri.MriCartesianOperator()
    op.setCoilSens(d["sens"])
    op.setMask(d["mask"])
    ref = CartesianCufft(d["sens"], d["mask"], roos, torch)
    stream = torch.cuda.current_stream()
    fwd = torch.empty((C, H, W), dtype=torch.complex64, device="cuda")
    adj = torch.empty((Hi, W), dtype=torch.complex64, device="cuda")
    op.forward(d["u"], out=fwd, stream=stream)
    op.adjoint(d["k"], out=adj, stream=stream)
    torch.cuda.synchronize()
    assert rel_l2(fwd.cpu().numpy(), ref.forward(d["u"]).cpu().numpy()) <= TOL
    assert rel_l2(adj.cpu().numpy(), ref.adjoint(d["k"]).cpu().numpy()) <= TOL


def test_iteration_operator_half_beside_cufft(pdt):
    """K^H of the k-space dual after one prox step, from the TGV-MRI solver's first iteration, against the
    cuFFT chain applied to the same ubar = u0 (config 2 shape, 15 coils x 640 x 368, ROOS)."""
    import torch

    from primaldualtoolbox.cufft_companion import CartesianCufft

    C, H, W = 15, 640, 368
    rng, sens, mask = _case(C, H, W, 7)
    d = {n: torch.from_numpy(a).cuda() for n, a in (("sens", sens), ("mask", mask))}
    ref = CartesianCufft(d["sens"], d["mask"], True, torch)
    u_true = (rng.standard_normal((H // 2, W)) + 1j * rng.standard_normal((H // 2, W))).astype(np.complex64)
    f = ref.forward(torch.from_numpy(u_true).cuda())
    op = pdt.mri.MriCartesianRemoveROOSOperator()
    op.setCoilSens(d["sens"])
    op.setMask(d["mask"])
    stream = torch.cuda.current_stream()
    u0 = torch.empty((H // 2, W), dtype=torch.complex64, device="cuda")
    op.adjoint(f, out=u0, stream=stream)
    torch.cuda.synchronize()
    assert rel_l2(u0.cpu().numpy(), ref.adjoint(f).cpu().numpy()) <= TOL
    sigma, lam = 0.125, 1.0
    r, khr = ref.prox_step(u0, torch.zeros_like(f), f, sigma, lam)
    ours_k = torch.empty_like(f)
    op.forward(u0, out=ours_k, stream=stream)
    ours_r = (sigma * (ours_k - f)) / (1.0 + sigma * lam)
    ours_khr = torch.empty_like(u0)
    op.adjoint(ours_r, out=ours_khr, stream=stream)
    torch.cuda.synchronize()
    assert rel_l2(ours_r.cpu().numpy(), r.cpu().numpy()) <= TOL
    assert rel_l2(ours_khr.cpu().numpy(), khr.cpu().numpy()) <= TOL
