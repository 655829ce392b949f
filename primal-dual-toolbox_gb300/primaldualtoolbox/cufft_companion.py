"""cuFFT companion of the Cartesian MRI operator: the reference's launch sequence restated on torch.fft.

The reference applies its Cartesian operators as a chain of separate launches around a batched cuFFT
2-D transform (mricartesianoperator.cu:196-265 plain, :320-414 ROOS):

  forward: padFOV (ROOS) -> prefft (sens_c . u, ifftshift with mid = int((n + 1) / 2)) -> fft2 with
           1/sqrt(W H) scaling -> fftshift2 (mid = n / 2) -> mask
  adjoint: preifft (mask, ifftshift) -> ifft2 -> fftshift2 -> combineImg (sum_c conj(sens_c) .) -> cropFOV

This module runs that same chain with torch.fft (cuFFT) on device tensors. It is a check and a timing
companion for the hand-written fused FFT kernels of libpdt.so: the tests compare the two operators on the
same inputs and bench.py times them side by side. No solver calls it.

Shapes follow the Python API: sens and k-space (C, H, W), mask (H, W), image (H, W) or (H / 2, W) with
ROOS removal (image rows at [y0, y0 + H / 2) of the H-row field, y0 = int(0.25 H + 1),
mricartesianoperator.cu:341).
"""
from __future__ import annotations

import numpy as np


def _mid_ifftshift(n):
    return int((float(n) + 1.0) / 2.0)


def roos_offset(H):
    """First field row of the ROOS image: `unsigned int FE_idx = size[1] * 0.25f + 1;` (float arithmetic)."""
    return int(np.float32(H) * np.float32(0.25) + np.float32(1.0))


class CartesianCufft:
    """Cartesian multi-coil operator (+ROOS) on cuFFT. sens (C, H, W) complex64, mask (H, W) float32."""

    def __init__(self, sens, mask, roos, torch):
        self.torch = torch
        self.sens = sens
        self.mask = mask
        self.roos = bool(roos)
        C, H, W = sens.shape
        self.C, self.H, self.W = C, H, W
        self.Hi = H // 2 if self.roos else H
        self.y0 = roos_offset(H) if self.roos else 0
        self.shift_in = (_mid_ifftshift(H), _mid_ifftshift(W))
        self.shift_out = (H // 2, W // 2)

    def forward(self, u):
        torch = self.torch
        if self.roos:
            img = torch.zeros((self.H, self.W), dtype=u.dtype, device=u.device)
            img[self.y0:self.y0 + self.Hi] = u
        else:
            img = u
        v = torch.roll(self.sens * img, shifts=self.shift_in, dims=(1, 2))
        k = torch.fft.fft2(v, norm="ortho")
        return torch.roll(k, shifts=self.shift_out, dims=(1, 2)) * self.mask

    def adjoint(self, k):
        torch = self.torch
        v = torch.roll(k * self.mask, shifts=self.shift_in, dims=(1, 2))
        g = torch.roll(torch.fft.ifft2(v, norm="ortho"), shifts=self.shift_out, dims=(1, 2))
        s = (torch.conj(self.sens) * g).sum(dim=0)
        return s[self.y0:self.y0 + self.Hi] if self.roos else s

    def prox_step(self, ubar, r, f, sigma, lam):
        """One operator half of a TGV-MRI iteration in the reference order (tgvmrioptimizer.cu:163-188):
        r <- (r + sigma (K ubar - f)) / (1 + sigma lambda), then K^H r. Returns (r, K^H r)."""
        r = (r + sigma * (self.forward(ubar) - f)) / (1.0 + sigma * lam)
        return r, self.adjoint(r)
