"""pdt_cartesian_forward_noalloc: the Cartesian forward operator for callers that cannot allocate
device memory (framework-owned memory pools, fixed memory budgets, allocator-free real-time loops).

It is called here through the C ABI with caller-owned device buffers and compared with the regular
operator entry point (pdt_op_forward) on two calls in a row, the second with new inputs and a different
size, so a stale scratch array from the first call would show. Tolerance: the operator parity bar,
rel-L2 <= 1e-5. This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

OP_TOL = 1e-5


def _case(rng, C, H, W, roos):
    sens = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
    mask = (rng.random((H, W)) < 0.5).astype(np.float32)
    Hi = H // 2 if roos else H
    img = (rng.standard_normal((Hi, W)) + 1j * rng.standard_normal((Hi, W))).astype(np.complex64)
    return sens, mask, img


def _regular_forward(pdt, roos, sens, mask, img):
    op = (pdt.mri.MriCartesianRemoveROOSOperator if roos else pdt.mri.MriCartesianOperator)()
    op.setCoilSens(sens)
    op.setMask(mask)
    return op.forward(img)


def test_noalloc_forward_matches_regular_entry_point(pdt):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox import _lib

    rng = np.random.default_rng(11)
    calls = [(True, 15, 640, 368), (False, 3, 48, 40)]
    for roos, C, H, W in calls:
        sens, mask, img = _case(rng, C, H, W, roos)
        d_sens = torch.from_numpy(sens).cuda()
        d_mask = torch.from_numpy(mask).cuda()
        d_img = torch.from_numpy(img).cuda()
        d_out = torch.full((C, H, W), float("nan"), dtype=torch.complex64, device="cuda")
        st = _lib.lib.pdt_cartesian_forward_noalloc(int(roos), ctypes.c_void_p(d_sens.data_ptr()),
                                                    ctypes.c_void_p(d_mask.data_ptr()), W, H, C,
                                                    ctypes.c_void_p(d_img.data_ptr()),
                                                    ctypes.c_void_p(d_out.data_ptr()), None)
        _lib.check(st)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        want = _regular_forward(pdt, roos, sens, mask, img)
        assert np.isfinite(got).all()
        assert rel_l2(got, want) <= OP_TOL


def test_noalloc_rejects_sizes_beyond_the_scratch(pdt):
    torch = pytest.importorskip("torch")
    from primaldualtoolbox import _lib

    d = torch.zeros(16, dtype=torch.complex64, device="cuda")
    # 64 coils x 1024 x 1024 image rows: 512 MiB of scratch, far above the 32 MiB limit
    st = _lib.lib.pdt_cartesian_forward_noalloc(0, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                                1024, 1024, 64, ctypes.c_void_p(d.data_ptr()),
                                                ctypes.c_void_p(d.data_ptr()), None)
    assert _lib.STATUS_NAMES[st] == "PDT_ERR_UNSUPPORTED"
    assert "static scratch" in _lib.lib.pdt_last_error().decode()
