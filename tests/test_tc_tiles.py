"""The tensor-core row passes' DFT-factor tables (pdt_cart_tiles.h), built on the host exactly as the operator
builds them (tests/native/tiles_emu.cpp), checked (1) bit for bit against a restatement of their layout:
2 x 2 real blocks of exp(+2 pi i p_s q(x) / W) (adjoint) or exp(-2 pi i q(x) f_s / W) (forward), 128-byte
swizzle of the 16-byte chunks, TF32 hi/lo split; and (2) as operators: the un-swizzled hi + lo factor
applied to random data gives the pruned DFT along W that the row pass computes, to FP32 accuracy."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

# (W, sampled columns, range rows NB): the benchmark geometry at 3 and 4 ranges, partial last ranges, a
# single chunk with one sampled column, every column sampled
GEOMS = [(368, 92, 256), (368, 92, 192), (48, 14, 32), (16, 5, 16), (320, 64, 224), (640, 200, 256),
         (96, 33, 64), (64, 1, 48), (32, 32, 64)]


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("tiles") / "tiles_emu.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", out,
                           os.path.join(HERE, "native", "tiles_emu.cpp")])
    lib = ctypes.CDLL(out)
    lib.emu_adj_table.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                  ctypes.c_longlong]
    lib.emu_adj_table.restype = ctypes.c_longlong
    lib.emu_fwd_table.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]
    lib.emu_fwd_table.restype = ctypes.c_longlong
    lib.emu_roots.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    return lib


def _tf32(v):
    u = np.ascontiguousarray(v, dtype=np.float32).view(np.uint32)
    return ((u + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)


def _case(emu, W, ns, NB):
    rng = np.random.default_rng(W * 31 + ns)
    cols = np.sort(rng.choice(W, ns, replace=False)).astype(np.int32)
    nch = (2 * ns + 31) // 32
    nranges = -(-2 * W // NB)
    size = nranges * nch * 2 * NB * 32
    out = np.full(size, np.nan, dtype=np.float32)
    assert emu.emu_adj_table(W, ns, cols.ctypes.data, NB, out.ctypes.data, size) == size
    roots = []
    for which in (0, 1):
        r = np.empty(W, dtype=np.float64)
        emu.emu_roots(W, which, r.ctypes.data)
        roots.append(r)
    return cols, out.reshape(nranges, nch, 2 * NB * 32), roots


def _restated(W, ns, cols, NB, cosr, sinr):
    """The table from its definition, one (range, chunk) block at a time."""
    nch, nranges = (2 * ns + 31) // 32, -(-2 * W // NB)
    mxW, oxW = (W + 1) // 2, W // 2
    wc, ws = cosr.astype(np.float32), sinr.astype(np.float32)
    tab = np.zeros((nranges, nch, 2 * NB * 32), dtype=np.float32)
    k = np.arange(32)
    for i in range(nranges):
        n0 = i * NB
        nb = min(NB, (2 * W - n0 + 15) & ~15)
        n = np.arange(nb)
        x, o = (n0 + n) >> 1, (n0 + n) & 1
        for j in range(nch):
            s, ri = 16 * j + (k >> 1), k & 1
            valid = (x[:, None] < W) & (s[None, :] < ns)
            p = (cols[np.minimum(s, ns - 1)].astype(np.int64) + mxW) % W
            q = (x.astype(np.int64) - oxW) % W
            m = (q[:, None] * p[None, :]) % W
            er, ei = wc[m], ws[m]
            v = np.where(o[:, None] == 0, np.where(ri[None, :] == 0, er, -ei), np.where(ri[None, :] == 0, ei, er))
            v = np.where(valid, v, np.float32(0)).astype(np.float32)
            hi = _tf32(v)
            lo = _tf32(v - hi)
            pos = (((k[None, :] >> 2) ^ (n[:, None] & 7)) << 2) + (k[None, :] & 3)
            H = np.zeros((nb, 32), dtype=np.float32)
            L = np.zeros((nb, 32), dtype=np.float32)
            np.put_along_axis(H, pos, hi, axis=1)
            np.put_along_axis(L, pos, lo, axis=1)
            tab[i, j, :nb * 32] = H.ravel()
            tab[i, j, nb * 32:2 * nb * 32] = L.ravel()
    return tab


@pytest.mark.parametrize("W,ns,NB", GEOMS)
def test_table_matches_its_layout_bit_for_bit(emu, W, ns, NB):
    cols, tab, (cosr, sinr) = _case(emu, W, ns, NB)
    want = _restated(W, ns, cols, NB, cosr, sinr)
    assert np.array_equal(tab.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("W,ns,NB", GEOMS)
def test_table_computes_the_pruned_inverse_dft(emu, W, ns, NB):
    cols, tab, _ = _case(emu, W, ns, NB)
    nch = tab.shape[1]
    # un-swizzle hi + lo into the real factor B[n][k] (n = 2 x + o output part, k = 2 s + ri input part)
    B = np.zeros((tab.shape[0] * NB, nch * 32))
    k = np.arange(32)
    for i in range(tab.shape[0]):
        nb = min(NB, (2 * W - i * NB + 15) & ~15)
        for j in range(nch):
            blk = tab[i, j].astype(np.float64)
            for n in range(nb):
                pos = (((k >> 2) ^ (n & 7)) << 2) + (k & 3)
                B[i * NB + n, 32 * j:32 * j + 32] = blk[n * 32 + pos] + blk[(nb + n) * 32 + pos]
    B = B[:2 * W, :2 * ns]
    rng = np.random.default_rng(W + ns)
    t2 = rng.standard_normal((7, ns)) + 1j * rng.standard_normal((7, ns))
    A = np.empty((7, 2 * ns))
    A[:, 0::2], A[:, 1::2] = t2.real, t2.imag
    D = A @ B.T
    g = D[:, 0::2] + 1j * D[:, 1::2]
    p = (cols.astype(np.int64) + (W + 1) // 2) % W
    q = (np.arange(W) - W // 2) % W
    want = t2 @ np.exp(2j * np.pi * np.outer(p, q) / W)
    assert np.linalg.norm(g - want) / np.linalg.norm(want) < 2e-7


# (W, sampled columns): one s tile, a partial s tile, several s tiles (ns > 128), W not a multiple of 16
FWD_GEOMS = [(368, 92), (48, 14), (16, 5), (320, 140), (640, 300), (100, 37), (64, 1)]


def _fwd_case(emu, W, ns):
    rng = np.random.default_rng(W * 17 + ns)
    cols = np.sort(rng.choice(W, ns, replace=False)).astype(np.int32)
    nchT, stiles, nbmax = (2 * W + 31) // 32, (ns + 127) // 128, (2 * min(128, ns) + 15) & ~15
    size = stiles * nchT * 2 * nbmax * 32
    out = np.full(size, np.nan, dtype=np.float32)
    assert emu.emu_fwd_table(W, ns, cols.ctypes.data, out.ctypes.data, size) == size
    return cols, out.reshape(stiles, nchT, 2 * nbmax * 32), nbmax


@pytest.mark.parametrize("W,ns", FWD_GEOMS)
def test_forward_table_matches_its_layout_bit_for_bit(emu, W, ns):
    cols, tab, nbmax = _fwd_case(emu, W, ns)
    r = [np.empty(W, dtype=np.float64) for _ in range(2)]
    for which in (0, 1):
        emu.emu_roots(W, which, r[which].ctypes.data)
    wc, ws = r[0].astype(np.float32), r[1].astype(np.float32)
    mxW, oxW = (W + 1) // 2, W // 2
    k = np.arange(32)
    for z in range(tab.shape[0]):
        nsl = min(128, ns - 128 * z)
        nb = (2 * nsl + 15) & ~15
        n = np.arange(2 * nsl)
        s, o = 128 * z + (n >> 1), n & 1
        f = (cols[s].astype(np.int64) - oxW) % W
        for j in range(tab.shape[1]):
            x, ri = 16 * j + (k >> 1), k & 1
            valid = np.broadcast_to(x[None, :] < W, (len(n), 32))
            q = (np.minimum(x, W - 1).astype(np.int64) + mxW) % W
            m = (f[:, None] * q[None, :]) % W
            er, ei = wc[m], -ws[m]
            v = np.where(o[:, None] == 0, np.where(ri[None, :] == 0, er, -ei), np.where(ri[None, :] == 0, ei, er))
            v = np.where(valid, v, np.float32(0)).astype(np.float32)
            hi = _tf32(v)
            lo = _tf32(v - hi)
            pos = (((k[None, :] >> 2) ^ (n[:, None] & 7)) << 2) + (k[None, :] & 3)
            H = np.zeros((len(n), 32), dtype=np.float32)
            L = np.zeros((len(n), 32), dtype=np.float32)
            np.put_along_axis(H, pos, hi, axis=1)
            np.put_along_axis(L, pos, lo, axis=1)
            want = np.zeros(2 * nbmax * 32, dtype=np.float32)
            want[:len(n) * 32] = H.ravel()
            want[nb * 32:nb * 32 + len(n) * 32] = L.ravel()
            assert np.array_equal(tab[z, j].view(np.uint32), want.view(np.uint32)), (z, j)


@pytest.mark.parametrize("W,ns", FWD_GEOMS)
def test_forward_table_computes_the_pruned_dft(emu, W, ns):
    cols, tab, nbmax = _fwd_case(emu, W, ns)
    nchT = tab.shape[1]
    B = np.zeros((2 * ns, nchT * 32))  # B[n][k]: n = 2 s + o output part, k = 2 x + ri input part
    k = np.arange(32)
    for z in range(tab.shape[0]):
        nsl = min(128, ns - 128 * z)
        nb = (2 * nsl + 15) & ~15
        for j in range(nchT):
            blk = tab[z, j].astype(np.float64)
            for n in range(2 * nsl):
                pos = (((k >> 2) ^ (n & 7)) << 2) + (k & 3)
                B[256 * z + n, 32 * j:32 * j + 32] = blk[n * 32 + pos] + blk[(nb + n) * 32 + pos]
    B = B[:, :2 * W]
    rng = np.random.default_rng(W + 3 * ns)
    a = rng.standard_normal((5, W)) + 1j * rng.standard_normal((5, W))
    A = np.empty((5, 2 * W))
    A[:, 0::2], A[:, 1::2] = a.real, a.imag
    D = A @ B.T
    t1 = D[:, 0::2] + 1j * D[:, 1::2]
    q = (np.arange(W) + (W + 1) // 2) % W
    f = (cols.astype(np.int64) - W // 2) % W
    want = a @ np.exp(-2j * np.pi * np.outer(q, f) / W)
    assert np.linalg.norm(t1 - want) / np.linalg.norm(want) < 2e-7
