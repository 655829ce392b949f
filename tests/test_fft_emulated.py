"""The engine's device FFT (pdt_device.cuh) compiled for the host with a one-thread emulation of the
block (tests/native/fft_emu.cpp) and checked against numpy: plan factorisation, twiddles, every
butterfly (radix 2, 3, 4, 5, 8, compile-time primes, runtime primes) and the Stockham index maps."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fftemu") / "fft_emu.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-o", out,
                           os.path.join(HERE, "native", "fft_emu.cpp")])
    lib = ctypes.CDLL(out)
    lib.emu_fft.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    return lib


SIZES = [1, 2, 3, 4, 5, 6, 7, 8, 10, 11, 13, 16, 17, 19, 23, 29, 31, 37, 46, 64, 96, 128, 192, 256, 320, 368, 384,
         640, 768, 1000, 2 * 41]


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("inverse", [0, 1])
def test_device_fft_matches_numpy(emu, n, inverse):
    rng = np.random.default_rng(n + 7 * inverse)
    x = (rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))).astype(np.complex64)
    y = x.copy()
    assert emu.emu_fft(y.ctypes.data, n, 3, inverse) == 0
    x64 = x.astype(np.complex128)
    ref = np.fft.ifft(x64, axis=1) * n if inverse else np.fft.fft(x64, axis=1)
    err = np.abs(y - ref).max() / np.abs(ref).max()
    assert err < 2e-6 * max(1.0, np.log2(max(n, 2)))


REG_SIZES = [2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 16, 20, 23, 24, 32]


@pytest.mark.parametrize("n", REG_SIZES)
@pytest.mark.parametrize("inverse", [0, 1])
def test_register_fft_matches_numpy(emu, n, inverse):
    emu.emu_regfft.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(100 + n)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    y = x.copy()
    assert emu.emu_regfft(y.ctypes.data, n, inverse) == 0
    x64 = x.astype(np.complex128)
    ref = np.fft.ifft(x64) * n if inverse else np.fft.fft(x64)
    assert np.abs(y - ref).max() / np.abs(ref).max() < 3e-6


TWO_LEVEL = [(16, 23), (32, 20), (16, 20), (16, 16), (12, 16), (16, 24), (8, 8), (16, 12), (8, 16), (32, 24),
             (16, 32), (8, 12), (8, 20)]


@pytest.mark.parametrize("ab", TWO_LEVEL)
@pytest.mark.parametrize("inverse", [0, 1])
def test_two_level_fft_matches_numpy(emu, ab, inverse):
    a, b = ab
    n = a * b
    emu.emu_twolevel.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(n + inverse)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    y = x.copy()
    assert emu.emu_twolevel(y.ctypes.data, a, b, inverse) == 0
    x64 = x.astype(np.complex128)
    ref = np.fft.ifft(x64) * n if inverse else np.fft.fft(x64)
    assert np.abs(y - ref).max() / np.abs(ref).max() < 5e-6


# (M, L) of every lane-FFT split the Cartesian kernels compile (n = M L), including both splits of 368
LANE_SPLITS = [(4, 8), (6, 8), (8, 8), (6, 16), (8, 16), (12, 16), (16, 16), (10, 32), (46, 8), (23, 16), (12, 32),
               (16, 32), (20, 32), (24, 32)]


@pytest.mark.parametrize("ml", LANE_SPLITS)
@pytest.mark.parametrize("inverse", [0, 1])
def test_lane_fft_matches_numpy(emu, ml, inverse):
    """LaneFft<M, L> with one host thread per lane: the M-point register FFT, the twiddle and the log2 L
    exchange stages, against numpy (forward; unnormalised inverse)."""
    m, l = ml
    n = m * l
    emu.emu_lanefft.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(3 * n + inverse)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    y = x.copy()
    assert emu.emu_lanefft(y.ctypes.data, m, l, inverse) == 0
    x64 = x.astype(np.complex128)
    ref = np.fft.ifft(x64) * n if inverse else np.fft.fft(x64)
    assert np.abs(y - ref).max() / np.abs(ref).max() < 5e-6


@pytest.mark.parametrize("m", [10, 6])
@pytest.mark.parametrize("inverse", [0, 1])
def test_two_warp_lane_fft_matches_numpy(emu, m, inverse):
    """LaneFft64<M> (n = 64 M over two warps; 640 = 10 x 64 is the readout-length column transform): the
    cross-warp stage through the shared buffer between 64-thread barriers, the rest as shuffles."""
    n = 64 * m
    emu.emu_lanefft64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(5 * n + inverse)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    y = x.copy()
    assert emu.emu_lanefft64(y.ctypes.data, m, inverse) == 0
    x64 = x.astype(np.complex128)
    ref = np.fft.ifft(x64) * n if inverse else np.fft.fft(x64)
    assert np.abs(y - ref).max() / np.abs(ref).max() < 5e-6
