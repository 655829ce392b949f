"""Seeded synthetic inputs with the shapes and statistics of the reference's workloads.

The reference's own knee/brain raw data and coil sensitivities are not distributed with it, so
benchmarks and tests use these generators instead (numpy only, deterministic per seed):

* ``tv_phantom``      piecewise-constant image of random ellipses / rectangles plus Gaussian noise
* ``mri_phantom``     complex Shepp-Logan-style phantom with a smooth random phase
* ``coil_maps``       Gaussian-blob coil sensitivities on a ring with random phase, sum |c|^2 = 1
* ``line_mask``       Cartesian phase-encode line mask (random or regular) with fully sampled centre
* ``cartesian_case``  all of the above plus noisy k-space for the (ROOS) Cartesian operator

The acquisition model here (``cartesian_forward`` / ``cartesian_adjoint``) is numpy's FFT with the
reference operator's shift conventions for even sizes (mricartesianoperator.cu:196-414); it only
synthesises data and is not used by the engine.
"""
from __future__ import annotations

import numpy as np


def tv_phantom(H=512, W=512, n_shapes=20, noise=0.1, seed=0):
    """float32 (H, W): n_shapes random ellipses/rectangles with intensities U(0,1), + N(0, noise^2)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    img = np.zeros((H, W))
    for _ in range(n_shapes):
        cy, cx = rng.uniform(0, H), rng.uniform(0, W)
        ry, rx = rng.uniform(0.03, 0.25) * H, rng.uniform(0.03, 0.25) * W
        val = rng.uniform(0, 1)
        if rng.uniform() < 0.5:
            th = rng.uniform(0, np.pi)
            dy, dx = y - cy, x - cx
            a = (dx * np.cos(th) + dy * np.sin(th)) / rx
            b = (-dx * np.sin(th) + dy * np.cos(th)) / ry
            inside = a * a + b * b <= 1
        else:
            inside = (np.abs(y - cy) <= ry) & (np.abs(x - cx) <= rx)
        img[inside] = val
    clean = img.astype(np.float32)
    noisy = (img + noise * rng.standard_normal((H, W))).astype(np.float32)
    return noisy, clean


# (intensity, semi-axis a, semi-axis b, centre x, centre y, angle in degrees) on [-1, 1]^2:
# the modified Shepp-Logan head phantom (Toft's contrast-enhanced variant of Shepp & Logan, 1974).
_SHEPP_LOGAN = [
    (1.0, 0.69, 0.92, 0.0, 0.0, 0),
    (-0.8, 0.6624, 0.874, 0.0, -0.0184, 0),
    (-0.2, 0.11, 0.31, 0.22, 0.0, -18),
    (-0.2, 0.16, 0.41, -0.22, 0.0, 18),
    (0.1, 0.21, 0.25, 0.0, 0.35, 0),
    (0.1, 0.046, 0.046, 0.0, 0.1, 0),
    (0.1, 0.046, 0.046, 0.0, -0.1, 0),
    (0.1, 0.046, 0.023, -0.08, -0.605, 0),
    (0.1, 0.023, 0.023, 0.0, -0.606, 0),
    (0.1, 0.023, 0.046, 0.06, -0.605, 0),
]


def mri_phantom(H=320, W=368, seed=0, phase_order=2):
    """complex64 (H, W) Shepp-Logan-style magnitude with a smooth random polynomial phase."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    # fit the head into the field of view, keeping its aspect ratio
    s = 0.95 * min(H, W) / 2
    X = (xx - (W - 1) / 2) / s
    Y = ((H - 1) / 2 - yy) / s
    img = np.zeros((H, W))
    for inten, a, b, x0, y0, ang in _SHEPP_LOGAN:
        t = np.deg2rad(ang)
        xr = (X - x0) * np.cos(t) + (Y - y0) * np.sin(t)
        yr = -(X - x0) * np.sin(t) + (Y - y0) * np.cos(t)
        img[(xr / a) ** 2 + (yr / b) ** 2 <= 1] += inten
    phase = np.zeros((H, W))
    for i in range(phase_order + 1):
        for j in range(phase_order + 1 - i):
            phase += rng.uniform(-1, 1) * (X / 1.5) ** i * (Y / 1.5) ** j
    return (img * np.exp(1j * np.pi * phase)).astype(np.complex64)


def coil_maps(C=15, H=640, W=368, seed=0, ring=0.55, width=0.45):
    """complex64 (C, H, W): Gaussian blobs centred on a ring, random phase, normalised to sum |c|^2 = 1."""
    rng = np.random.default_rng(seed + 1000)
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    Y = (yy - H / 2) / (H / 2)
    X = (xx - W / 2) / (W / 2)
    maps = np.empty((C, H, W), dtype=np.complex128)
    for c in range(C):
        ang = 2 * np.pi * c / C + rng.uniform(-0.1, 0.1)
        cy, cx = ring * np.sin(ang), ring * np.cos(ang)
        mag = np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * width ** 2))
        ph = rng.uniform(0, 2 * np.pi) + rng.uniform(-1, 1) * X + rng.uniform(-1, 1) * Y
        maps[c] = mag * np.exp(1j * ph)
    maps /= np.sqrt(np.sum(np.abs(maps) ** 2, axis=0, keepdims=True))
    return maps.astype(np.complex64)


def line_mask(H=640, W=368, accel=4, center=28, seed=0, kind="random"):
    """float32 (H, W) mask of fully sampled phase-encode lines (columns): `center` central lines plus
    random (or regularly spaced) lines up to W/accel in total."""
    rng = np.random.default_rng(seed + 2000)
    n_total = max(int(round(W / accel)), min(center, W))
    cols = set(range(max(0, W // 2 - center // 2), min(W, W // 2 - center // 2 + center)))
    if kind == "regular":
        cols |= set(range(0, W, int(accel)))
    else:
        rest = np.array([c for c in range(W) if c not in cols])
        need = max(0, n_total - len(cols))
        if need and len(rest):
            cols |= set(rng.choice(rest, size=min(need, len(rest)), replace=False).tolist())
    m = np.zeros((H, W), dtype=np.float32)
    m[:, sorted(cols)] = 1
    return m


def roos_offset(H_full):
    """First image row inside the oversampled readout FOV: unsigned(H * 0.25f + 1) as the reference."""
    return int(np.float32(H_full) * np.float32(0.25) + np.float32(1))


def cartesian_forward(img, sens, mask, roos):
    C, Hf, W = sens.shape
    x = img
    if roos:
        x = np.zeros((Hf, W), dtype=np.complex128)
        y0 = roos_offset(Hf)
        x[y0:y0 + img.shape[0]] = img
    k = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(sens * x[None], axes=(-2, -1)), norm="ortho"), axes=(-2, -1))
    return k * mask[None]


def cartesian_adjoint(k, sens, mask, roos):
    C, Hf, W = sens.shape
    g = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(k * mask[None], axes=(-2, -1)), norm="ortho"), axes=(-2, -1))
    x = np.sum(np.conj(sens) * g, axis=0)
    if roos:
        y0 = roos_offset(Hf)
        x = x[y0:y0 + Hf // 2]
    return x


def cartesian_case(C=15, H=640, W=368, roos=True, accel=4, center=28, mask_kind="random", noise=1e-3, seed=0,
                   alpha_scale=0.05):
    """A synthetic Cartesian multi-coil reconstruction problem.

    Returns a dict with rawdata (C, H, W) c64, sens (C, H, W) c64, mask (H, W) f32, truth (H/2 or H, W) c64,
    alpha1 = alpha_scale * max|K^H f| and alpha0 = 2 alpha1 (the sample's alpha0 = 2 alpha1).
    """
    Hi = H // 2 if roos else H
    truth = mri_phantom(Hi, W, seed=seed)
    sens = coil_maps(C, H, W, seed=seed)
    mask = line_mask(H, W, accel=accel, center=center, seed=seed, kind=mask_kind)
    k = cartesian_forward(truth.astype(np.complex128), sens.astype(np.complex128), mask, roos)
    rng = np.random.default_rng(seed + 3000)
    sigma = noise * np.abs(k).max()
    k = k + mask[None] * sigma * (rng.standard_normal(k.shape) + 1j * rng.standard_normal(k.shape)) / np.sqrt(2)
    rawdata = k.astype(np.complex64)
    s = float(np.abs(cartesian_adjoint(rawdata.astype(np.complex128), sens, mask, roos)).max())
    alpha1 = alpha_scale * s
    return {"rawdata": rawdata, "sens": sens, "mask": mask, "truth": truth, "alpha1": alpha1,
            "alpha0": 2 * alpha1, "roos": roos}
