"""ctypes front-end of the CPU oracle (oracle/pdt_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the cpu_baseline /
reference legs of ``bench.py`` -- always as the checker or the timed CPU baseline, never as the product
path. The product (``primaldualtoolbox`` over ``libpdt.so``) never imports this module.

Array conventions follow the reference's Python bindings (python/pyMriReconstruction.cpp:39-93):
numpy arrays in C order, k-space ``(C, FE, PE)``, images ``(FE, PE)``, which is ImageUtilities'
``(PE, FE, C)`` with PE fastest.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")
_SRC = os.path.join(_HERE, "pdt_oracle.cpp")

KIND = {"cartesian": 0, "cartesian_roos": 1, "sampling": 2}
VARIANT = {"tgv_mri": 0, "tgv_op": 1, "tv_op": 2}


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (OpenMP, no FP contraction so x86 and Arm agree)."""
    os.makedirs(_BUILD, exist_ok=True)
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC):
        tmp = _LIB_PATH + ".tmp"
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
                               "-ffp-contract=off", "-o", tmp, _SRC])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, i, d, u = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint
        L.orc_fft1d.argtypes = [vp, i, i]
        L.orc_set_threads.argtypes = [i]
        L.orc_max_threads.restype = i
        L.orc_tv_solve.argtypes = [i, i, i, i, vp, vp, vp, d, u]
        L.orc_tgv_solve.argtypes = [i, i, i, i, vp, vp, vp, d, d, d, u]
        L.orc_op_apply.argtypes = [i, i, i, i, i, i, vp, vp, vp, vp]
        L.orc_op_solve.argtypes = [i, i, i, i, i, vp, vp, vp, vp, vp, i, d, d, d, d, u, vp, vp]
        L.orc_alpha_schedule_f32.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float, u, u,
                                             ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
        L.orc_radial_apply.argtypes = [i, i, i, d, i, i, i, vp, vp, vp, vp, vp]
        L.orc_radial_solve.argtypes = [i, i, d, i, i, i, vp, vp, vp, vp, vp, vp, i, d, d, d, d, u]
        L.orc_radial_grid_size.argtypes = [i, d]
        L.orc_radial_grid_size.restype = i
        L.orc_kb_beta.argtypes = [i, d]
        L.orc_kb_beta.restype = d
        L.orc_kb_deapod.argtypes = [i, i, i, d]
        L.orc_kb_deapod.restype = d
        L.orc_cnn_grad_exact.restype = d
        L.orc_cnn_grad_exact.argtypes = [i, i, i, vp, vp, vp, vp, vp]
        L.orc_cnn_grad.restype = d
        L.orc_cnn_grad.argtypes = [i, i, i, vp, vp, vp, vp, vp, vp]
        L.orc_tgv_energy_f64.restype = d
        L.orc_tgv_energy_f64.argtypes = [i, i, i, i, vp, vp, vp, vp, vp, vp, d, d]
        L.orc_op_gap.restype = None
        L.orc_op_gap.argtypes = [i, i, i, i, vp, vp, vp, vp, i, d, d, d, vp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _cx(prec):
    return np.complex64 if prec == 32 else np.complex128


def _re(prec):
    return np.float32 if prec == 32 else np.float64


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return lib().orc_max_threads()


def fft1d(x, inverse=False):
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    lib().orc_fft1d(_ptr(a), a.size, 1 if inverse else -1)
    return a


def op_apply(kind, sens, mask, src, adjoint=False, prec=64):
    """Forward (image -> k-space) or adjoint (k-space -> image) of a Cartesian-family operator."""
    k = KIND[kind]
    mask = np.ascontiguousarray(mask, dtype=_re(prec))
    Hf, W = mask.shape
    if k == 2:
        C, s = 1, None
    else:
        s = np.ascontiguousarray(sens, dtype=_cx(prec))
        C = s.shape[0]
    Hi = Hf // 2 if k == 1 else Hf
    src = np.ascontiguousarray(src, dtype=_cx(prec))
    if adjoint:
        dst = np.zeros((Hi, W), dtype=_cx(prec))
    else:
        dst = np.zeros((Hf, W) if k == 2 else (C, Hf, W), dtype=_cx(prec))
    lib().orc_op_apply(prec, k, int(adjoint), W, Hf, C, _ptr(s), _ptr(mask), _ptr(src), _ptr(dst))
    return dst


def op_solve(kind, sens, mask, f, variant="tgv_mri", alpha0=1.0, alpha1=1.0, reduction=1.0, lam=1.0,
             max_iter=1, u0=None, prec=32, return_state=False, state=None):
    """TgvMriOptimizer / TgvOptimizerWithOp / TvOptimizerWithOp with a Cartesian-family operator.
    `state` (a dict as returned with return_state=True) continues a previous solve from all of its
    primal and dual variables, as a second solve() call on the same optimizer does."""
    k = KIND[kind]
    mask = np.ascontiguousarray(mask, dtype=_re(prec))
    Hf, W = mask.shape
    if k == 2:
        C, s = 1, None
    else:
        s = np.ascontiguousarray(sens, dtype=_cx(prec))
        C = s.shape[0]
    Hi = Hf // 2 if k == 1 else Hf
    f = np.ascontiguousarray(f, dtype=_cx(prec))
    u0 = None if u0 is None else np.ascontiguousarray(u0, dtype=_cx(prec))
    u = np.zeros((Hi, W), dtype=_cx(prec))
    names = ["u", "ubar", "vx", "vy", "vbx", "vby", "px", "py", "qxx", "qyy", "qxy"]
    sin = None
    if state is not None:
        sin = np.concatenate([np.ravel(state[nm]) for nm in names] + [np.ravel(state["r"])]).astype(_cx(prec))
        if sin.size != 11 * Hi * W + C * Hf * W:
            raise ValueError("state does not match the problem size")
    state = np.zeros(11 * Hi * W + C * Hf * W, dtype=_cx(prec)) if return_state else None
    lib().orc_op_solve(prec, k, W, Hf, C, _ptr(s), _ptr(mask), _ptr(f), _ptr(u0), _ptr(u), VARIANT[variant],
                       alpha0, alpha1, reduction, lam, int(max_iter), _ptr(state), _ptr(sin))
    if return_state:
        n = Hi * W
        st = {nm: state[i * n:(i + 1) * n].reshape(Hi, W) for i, nm in enumerate(names)}
        st["r"] = state[11 * n:].reshape((Hf, W) if k == 2 else (C, Hf, W))
        return u, st
    return u


def tv_solve(f, lam=1.0, max_iter=1, u0=None, prec=32):
    cplx = np.iscomplexobj(f)
    dt = _cx(prec) if cplx else _re(prec)
    f = np.ascontiguousarray(f, dtype=dt)
    u0 = None if u0 is None else np.ascontiguousarray(u0, dtype=dt)
    u = np.zeros_like(f)
    H, W = f.shape
    lib().orc_tv_solve(prec, int(cplx), W, H, _ptr(f), _ptr(u0), _ptr(u), lam, int(max_iter))
    return u


def tgv_solve(f, lam=1.0, alpha0=1.0, alpha1=1.0, max_iter=1, u0=None, prec=32):
    cplx = np.iscomplexobj(f)
    dt = _cx(prec) if cplx else _re(prec)
    f = np.ascontiguousarray(f, dtype=dt)
    u0 = None if u0 is None else np.ascontiguousarray(u0, dtype=dt)
    u = np.zeros_like(f)
    H, W = f.shape
    lib().orc_tgv_solve(prec, int(cplx), W, H, _ptr(f), _ptr(u0), _ptr(u), lam, alpha0, alpha1, int(max_iter))
    return u


def alpha_schedule(alpha0, alpha1, reduction, max_iter, k):
    o0, o1 = ctypes.c_float(), ctypes.c_float()
    lib().orc_alpha_schedule_f32(alpha0, alpha1, reduction, int(max_iter), int(k), ctypes.byref(o0),
                                 ctypes.byref(o1))
    return o0.value, o1.value


def tgv_energy(kind, sens, mask, f, u, vx, vy, alpha0, alpha1):
    k = KIND[kind]
    mask = np.ascontiguousarray(mask, dtype=np.float64)
    Hf, W = mask.shape
    s = None if k == 2 else np.ascontiguousarray(sens, dtype=np.complex128)
    C = 1 if k == 2 else s.shape[0]
    arrs = [np.ascontiguousarray(a, dtype=np.complex128) for a in (f, u, vx, vy)]
    return lib().orc_tgv_energy_f64(k, W, Hf, C, _ptr(s), _ptr(mask), *[_ptr(a) for a in arrs], alpha0, alpha1)


STATE_NAMES = ["u", "ubar", "vx", "vy", "vbx", "vby", "px", "py", "qxx", "qyy", "qxy"]


def op_gap(kind, sens, mask, f, state, variant="tgv_mri", alpha0=1.0, alpha1=1.0, lam=1.0):
    """FP64 primal-dual gap and dual-constraint residuals of a with-operator state (op_solve's
    return_state dict): {'gap', 'primal', 'dual', 'residual_u', 'residual_v', 'norm_khr'}."""
    k = KIND[kind]
    mask = np.ascontiguousarray(mask, dtype=np.float64)
    Hf, W = mask.shape
    s = None if k == 2 else np.ascontiguousarray(sens, dtype=np.complex128)
    C = 1 if k == 2 else s.shape[0]
    f = np.ascontiguousarray(f, dtype=np.complex128)
    flat = np.concatenate([np.ravel(state[nm]) for nm in STATE_NAMES] + [np.ravel(state["r"])]).astype(np.complex128)
    out = np.zeros(6)
    lib().orc_op_gap(k, W, Hf, C, _ptr(s), _ptr(mask), _ptr(f), _ptr(flat), VARIANT[variant], alpha0, alpha1, lam,
                     _ptr(out))
    return dict(zip(("gap", "primal", "dual", "residual_u", "residual_v", "norm_khr"), out.tolist()))


def _radial_args(traj, dcf, sens, prec):
    traj = np.ascontiguousarray(traj, dtype=_re(prec)).reshape(2, -1)
    Ns = traj.shape[1]
    dcf = np.ascontiguousarray(dcf, dtype=_re(prec)).reshape(-1)
    assert dcf.size == Ns
    s = None if sens is None else np.ascontiguousarray(sens, dtype=_cx(prec))
    C = 1 if s is None else s.shape[0]
    return traj, dcf, s, C, Ns


def radial_apply(traj, dcf, sens, src, N, osf, kw, mode="forward", prec=64):
    """Radial multi-coil (sens (C,N,N)) or single-coil (sens None) operator. traj (2, Ns): row 0 pairs with
    image x, row 1 with y; dcf (1, Ns) or (Ns,). mode: forward | adjoint | ndft."""
    traj, dcf, s, C, Ns = _radial_args(traj, dcf, sens, prec)
    src = np.ascontiguousarray(src, dtype=_cx(prec))
    m = {"forward": 0, "adjoint": 1, "ndft": 2}[mode]
    dst = np.zeros((N, N) if m == 1 else (C, Ns), dtype=_cx(prec))
    lib().orc_radial_apply(prec, m, N, osf, kw, C, Ns, _ptr(traj), _ptr(dcf), _ptr(s), _ptr(src), _ptr(dst))
    return dst


def radial_solve(traj, dcf, sens, f, N, osf, kw, variant="tgv_mri", alpha0=1.0, alpha1=1.0, reduction=1.0, lam=1.0,
                 max_iter=1, u0=None, prec=32):
    traj, dcf, s, C, Ns = _radial_args(traj, dcf, sens, prec)
    f = np.ascontiguousarray(f, dtype=_cx(prec))
    u0 = None if u0 is None else np.ascontiguousarray(u0, dtype=_cx(prec))
    u = np.zeros((N, N), dtype=_cx(prec))
    lib().orc_radial_solve(prec, N, osf, kw, C, Ns, _ptr(traj), _ptr(dcf), _ptr(s), _ptr(f), _ptr(u0), _ptr(u),
                           VARIANT[variant], alpha0, alpha1, reduction, lam, int(max_iter))
    return u


def radial_grid_size(N, osf):
    return lib().orc_radial_grid_size(N, osf)


def cnn_grad(params, u0, ut, vt):
    """Loss, flat gradient (FP64) and output (B, H, W, 8) of the warm-start network for a batch.
    u0, ut: (B, H, W) complex64; vt: (B, 2, H, W) complex64; params: flat float32."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    u0 = np.ascontiguousarray(u0, dtype=np.complex64)
    ut = np.ascontiguousarray(ut, dtype=np.complex64)
    vt = np.ascontiguousarray(vt, dtype=np.complex64)
    B, H, W = u0.shape
    g = np.zeros(params.size, dtype=np.float64)
    out = np.zeros((B, H, W, 8), dtype=np.float64)
    loss = lib().orc_cnn_grad(B, H, W, _ptr(params), _ptr(u0), _ptr(ut), _ptr(vt), _ptr(g), _ptr(out))
    return loss, g, out


def cnn_grad_exact(params, u0, ut, vt):
    """Loss and gradient of the network in FP64 without BF16 rounding (finite-difference checkable)."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    u0, ut, vt = (np.ascontiguousarray(a, dtype=np.complex64) for a in (u0, ut, vt))
    B, H, W = u0.shape
    g = np.zeros(params.size, dtype=np.float64)
    loss = lib().orc_cnn_grad_exact(B, H, W, _ptr(params), _ptr(u0), _ptr(ut), _ptr(vt), _ptr(g))
    return loss, g
