"""ctypes front-end of oracle/_ref/libpdtref.so, the reference's own optimizer and Cartesian-operator sources
compiled for the CPU (oracle/ref_build.py, oracle/ref_driver.cpp).

TEST INFRASTRUCTURE ONLY: it pins the oracle restatement (oracle/pdt_oracle.cpp) in tests and writes the
golden vectors in tests/golden/. It exists only where the reference checkout is present (the library is
built from it); `available()` says whether it is. Arrays follow the reference's Python bindings: numpy
C order, k-space (C, FE, PE), images (FE, PE), complex64 / float32.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def available() -> bool:
    """Builds the library when the reference checkout exists; False where it does not."""
    from . import ref_build

    try:
        return ref_build.build() is not None
    except Exception:
        return False


def lib():
    global _lib
    if _lib is None:
        from . import ref_build

        path = ref_build.build()
        if path is None:
            raise RuntimeError("the reference checkout is not available: oracle/_ref cannot be built")
        L = ctypes.CDLL(path)
        vp, i, f, u = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_cart_apply.argtypes = [i, i, i, i, i, vp, vp, vp, vp]
        L.ref_tgv_mri.argtypes = [i, i, i, i, vp, vp, vp, vp, f, f, f, u, vp]
        L.ref_with_op.argtypes = [i, i, i, i, i, vp, vp, vp, f, f, f, u, vp]
        L.ref_denoise.argtypes = [i, i, i, i, vp, f, f, f, u, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(rc):
    if rc:
        raise RuntimeError(lib().ref_last_error().decode())


def _cart_args(sens, mask):
    sens = np.ascontiguousarray(sens, dtype=np.complex64)
    mask = np.ascontiguousarray(mask, dtype=np.float32)
    C, Hf, W = sens.shape
    return sens, mask, C, Hf, W


def cart_apply(roos, sens, mask, src, adjoint=False):
    """MriCartesian(RemoveROOS)Operator forward (image -> k-space) or adjoint."""
    sens, mask, C, Hf, W = _cart_args(sens, mask)
    src = np.ascontiguousarray(src, dtype=np.complex64)
    Hi = Hf // 2 if roos else Hf
    dst = np.zeros((Hi, W) if adjoint else (C, Hf, W), np.complex64)
    _check(lib().ref_cart_apply(int(roos), int(adjoint), W, Hf, C, _p(sens), _p(mask), _p(src), _p(dst)))
    return dst


def tgv_mri(roos, sens, mask, f, alpha0, alpha1, reduction, max_iter, u0=None):
    """TgvMriOptimizer_2c3c.solve(): max_iter + 1 iterations from u0 (default A^H f)."""
    sens, mask, C, Hf, W = _cart_args(sens, mask)
    f = np.ascontiguousarray(f, dtype=np.complex64)
    u0 = None if u0 is None else np.ascontiguousarray(u0, dtype=np.complex64)
    Hi = Hf // 2 if roos else Hf
    out = np.zeros((Hi, W), np.complex64)
    _check(lib().ref_tgv_mri(int(roos), W, Hf, C, _p(sens), _p(mask), _p(f), _p(u0), alpha0, alpha1, reduction,
                             int(max_iter), _p(out)))
    return out


def with_op(variant, roos, sens, mask, f, lam, max_iter, alpha0=1.0, alpha1=1.0):
    """TgvOptimizerWithOp ('tgv_op') or TvOptimizerWithOp ('tv_op') with a Cartesian operator."""
    sens, mask, C, Hf, W = _cart_args(sens, mask)
    f = np.ascontiguousarray(f, dtype=np.complex64)
    Hi = Hf // 2 if roos else Hf
    out = np.zeros((Hi, W), np.complex64)
    _check(lib().ref_with_op(0 if variant == "tgv_op" else 1, int(roos), W, Hf, C, _p(sens), _p(mask), _p(f), lam,
                             alpha0, alpha1, int(max_iter), _p(out)))
    return out


def denoise(kind, f, lam, max_iter, alpha0=1.0, alpha1=1.0):
    """TvOptimizer ('tv') or TgvOptimizer ('tgv') on a float32 or complex64 image."""
    cplx = np.iscomplexobj(f)
    f = np.ascontiguousarray(f, dtype=np.complex64 if cplx else np.float32)
    H, W = f.shape
    out = np.zeros_like(f)
    _check(lib().ref_denoise(1 if kind == "tgv" else 0, int(cplx), W, H, _p(f), lam, alpha0, alpha1, int(max_iter),
                             _p(out)))
    return out
