"""primaldualtoolbox.warmstart -- the learned warm start for TGV^2 MRI reconstruction.

A small residual CNN (8 convolutions, 32 channels, 3 x 3, BF16 weights / activations, FP32 accumulation;
libpdt.so's own tensor-core kernels for inference and training) maps the zero-filled image
u0 = A^H f to an initial (u, v). ``warm_start`` applies it to an optimizer and keeps the plain start
(u0, v = 0) whenever the network's start has the higher TGV energy -- the primal-dual iteration that
follows still decides the result.

Training data are made by the engine itself: converged TGV^2 solutions at fixed alpha of synthetic
Cartesian problems (``make_training_set``), solved many at a time with ``primaldualtoolbox.batch`` with the
dual-weighted step sizes ``DUAL_WEIGHTED_STEPS``, which reach the same saddle point as the reference's
steps 15-80 times sooner (8000 iterations: rel-L2 well below 1e-4 of the limit).

    python -m primaldualtoolbox.warmstart --shape 15,320,320 --roos 0 --cases 4096 --out weights.npz

There is no counterpart in the reference.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import time

import numpy as np

from . import _lib
from ._lib import Buffer, check, lib

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
DEFAULT_WEIGHTS = os.path.join(_DATA, "warmstart_15c_640x368.npz")
# the learned-warm-start configuration: 15 coils, 320 x 320, 4x
CONFIG4_WEIGHTS = os.path.join(_DATA, "warmstart_15c_320x320.npz")
# radial: 12 coils, 256 x 256, 64 golden-angle spokes x 512 samples, Kaiser-Bessel width 3, grid 1.5x
RADIAL_WEIGHTS = os.path.join(_DATA, "warmstart_radial_12c_256.npz")
RADIAL_GEOMETRY = dict(N=256, C=12, spokes=64, readout=512, osf=1.5, kernel_width=3)


def radial_trajectory(spokes=64, readout=512):
    """(2, spokes * readout) float32 golden-angle trajectory in the reference sample's layout (row 0 the
    imaginary, row 1 the real part of k, bin/mri_radial_test.py:38) and the density weights sqrt|k|."""
    ang = np.arange(spokes) * np.pi * (np.sqrt(5) - 1) / 2
    r = (np.arange(readout) - readout / 2) / readout
    k = (r[:, None] * np.exp(1j * ang[None, :])).ravel()
    return np.array([k.imag, k.real]).astype(np.float32), np.sqrt(np.abs(k)).astype(np.float32)[None, :]


def radial_problem(pdt, seed, torch=None, N=256, C=12, spokes=64, readout=512, osf=1.5, kernel_width=3,
                   noise=0.01, alpha_scale=0.02):
    """A seeded radial TGV-MRI problem: MriRadialOperator with seeded coil maps, data f = A(phantom) plus
    complex noise of `noise` x max|f|, alpha1 = alpha_scale x max|A^H f|. Returns (op, f, alpha1); f is a
    device tensor when torch is given."""
    from . import synthetic

    traj, dcf = radial_trajectory(spokes, readout)
    op = pdt.mri.MriRadialOperator({"osf": osf, "sector_width": 8, "kernel_width": kernel_width, "img_dim": N})
    op.setTrajectory(traj)
    op.setDcf(dcf)
    op.setCoilSens(synthetic.coil_maps(C, N, N, seed=seed))
    f = op.forward(synthetic.mri_phantom(N, N, seed=seed))
    rng = np.random.default_rng(seed)
    f = f + (noise * np.abs(f).max() * (rng.standard_normal(f.shape) + 1j * rng.standard_normal(f.shape))).astype(
        np.complex64)
    alpha1 = alpha_scale * float(np.abs(op.adjoint(f)).max())
    if torch is not None:
        f = torch.from_numpy(np.ascontiguousarray(f)).cuda()
    return op, f, alpha1


def make_radial_training_set(pdt, torch, n_cases, iters, seed0=1000, batch=16, log=print, steps=None):
    """(u0, u*, v*) of n_cases seeded radial problems (RADIAL_GEOMETRY), u* after `iters` iterations at
    fixed alpha with step sizes `steps` (None: the reference's), `batch` problems at a time."""
    N = RADIAL_GEOMETRY["N"]
    U0 = torch.empty((n_cases, N, N), dtype=torch.complex64, device="cuda")
    UT = torch.empty_like(U0)
    VT = torch.empty((n_cases, 2, N, N), dtype=torch.complex64, device="cuda")
    t0 = time.time()
    for start in range(0, n_cases, batch):
        opts, keep = [], []
        for i in range(start, min(n_cases, start + batch)):
            op, f, a1 = radial_problem(pdt, seed0 + i, torch)
            opt = pdt.mri.TgvMriOptimizer_2c2c()
            prm = opt.getParameters()
            prm.max_iter, prm.reduction, prm.alpha1, prm.alpha0 = iters - 1, 1.0, a1, 2 * a1
            if steps:
                opt.setSteps(*steps)
            opt.setOperator(op)
            opt.setNoisyData(f)
            op.adjoint(f, out=U0[i])
            opt.setInput0(U0[i])
            opts.append((i, opt))
            keep.append((op, f))
        pdt.batch.BatchSolver([o for _, o in opts]).solve()
        for i, opt in opts:
            opt.getResult(out=UT[i])
            opt.getField("vx", out=VT[i, 0])
            opt.getField("vy", out=VT[i, 1])
        torch.cuda.synchronize()
        log(f"targets {min(n_cases, start + batch)}/{n_cases}  {time.time() - t0:.1f}s")
    return U0, UT, VT

# (tau, sigma) of the dual-weighted solve: the same primal-dual iteration with tau sigma = 1/16 (the
# reference's TGV-MRI steps have tau sigma = 1/128; convergence needs tau sigma |K|^2 < 1, |K|^2 <= 13
# for TGV with a unit-norm operator) and sigma / tau = 1024 instead of 2. The fixed-alpha iteration's
# slow tail is the convergence of the duals p, q; this balance moves them 512 times faster relative to
# the primal, and the iteration reaches rel-L2 1e-4 of the same solution in thousands instead of
# hundreds of thousands of iterations.
DUAL_WEIGHTED_STEPS = (1.0 / 128.0, 8.0)


def dual_weighted_steps(op_norm=1.0, ratio=1024.0, margin=0.8):
    """(tau, sigma) with sigma / tau = ratio and tau sigma (12 + |K|^2) = margin for an operator of norm
    op_norm (12 bounds |[grad, -1; 0, eps]|^2 of the TGV part). For op_norm = 1 this is about
    DUAL_WEIGHTED_STEPS."""
    ts = margin / (12.0 + float(op_norm) ** 2)
    tau = (ts / ratio) ** 0.5
    return tau, ratio * tau


def _bind():
    vp, i = ctypes.c_void_p, ctypes.c_int
    lib.pdt_cnn_create.argtypes = [ctypes.c_uint64, ctypes.POINTER(vp)]
    lib.pdt_cnn_destroy.argtypes = [vp]
    lib.pdt_cnn_num_params.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
    lib.pdt_cnn_get_params.argtypes = [vp, vp, ctypes.c_size_t]
    lib.pdt_cnn_set_params.argtypes = [vp, vp, ctypes.c_size_t]
    lib.pdt_cnn_get_grads.argtypes = [vp, vp, ctypes.c_size_t]
    lib.pdt_cnn_train_step.argtypes = [vp, vp, vp, vp, i, i, i, ctypes.c_float, vp, ctypes.POINTER(ctypes.c_double)]
    lib.pdt_cnn_predict.argtypes = [vp, vp, i, i, i, vp, vp, vp]
    for n in ("pdt_cnn_create", "pdt_cnn_destroy", "pdt_cnn_num_params", "pdt_cnn_get_params", "pdt_cnn_set_params",
              "pdt_cnn_get_grads", "pdt_cnn_train_step", "pdt_cnn_predict"):
        getattr(lib, n).restype = ctypes.c_int


_bind()


def _dev(a, dtype):
    b = Buffer(a, dtype)
    if not b.is_device:
        raise TypeError("the network takes device arrays (e.g. torch CUDA tensors)")
    return b


class WarmStartNet:
    """The warm-start network. Images are device arrays: u0 (B, H, W) complex64, v (B, 2, H, W)."""

    def __init__(self, seed=0, weights=None):
        h = ctypes.c_void_p()
        check(lib.pdt_cnn_create(int(seed), ctypes.byref(h)))
        self._h = h
        if weights is not None:
            self.load(weights)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pdt_cnn_destroy(h)
            self._h = None

    @property
    def num_params(self):
        n = ctypes.c_size_t()
        check(lib.pdt_cnn_num_params(self._h, ctypes.byref(n)))
        return n.value

    def get_params(self):
        out = np.empty(self.num_params, dtype=np.float32)
        check(lib.pdt_cnn_get_params(self._h, out.ctypes.data, out.size))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib.pdt_cnn_set_params(self._h, p.ctypes.data, p.size))

    def grads(self):
        out = np.empty(self.num_params, dtype=np.float32)
        check(lib.pdt_cnn_get_grads(self._h, out.ctypes.data, out.size))
        return out

    def save(self, path, **meta):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez(path, params=self.get_params(), meta=json.dumps(meta))

    def load(self, path):
        with np.load(path) as z:
            self.set_params(z["params"])

    def train_step(self, u0, ut, vt, lr=1e-3, stream=None):
        """Forward, backward and (lr > 0) one Adam step; returns the loss (mean squared error per pixel)."""
        a, b, c = _dev(u0, np.complex64), _dev(ut, np.complex64), _dev(vt, np.complex64)
        B, H, W = a.shape
        loss = ctypes.c_double()
        check(lib.pdt_cnn_train_step(self._h, a.ptr, b.ptr, c.ptr, B, H, W, float(lr), _lib.stream_handle(stream),
                                     ctypes.byref(loss)))
        return loss.value

    def predict(self, u0, u_out, v_out, stream=None):
        a = _dev(u0, np.complex64)
        B, H, W = a.shape
        check(lib.pdt_cnn_predict(self._h, a.ptr, B, H, W, _dev(u_out, np.complex64).ptr,
                                  _dev(v_out, np.complex64).ptr, _lib.stream_handle(stream)))


def warm_start(optimizer, net, u0, torch, stream=None):
    """Starts `optimizer` (a TGV-MRI optimizer with operator and data set) from the network's (u, v) when
    that start has the lower FP64 TGV energy, else from the plain start (u0 = A^H f, v = 0). u0 is the
    device image A^H f, shape (H, W). Returns {'used': 'network' | 'plain', 'energy_network', 'energy_plain'}."""
    H, W = u0.shape
    u = torch.empty((1, H, W), dtype=torch.complex64, device=u0.device)
    v = torch.empty((1, 2, H, W), dtype=torch.complex64, device=u0.device)
    net.predict(u0.reshape(1, H, W), u, v, stream=stream)
    optimizer.setInput0(u0, stream=stream)
    e_plain = optimizer.energy(stream=stream)["total"]
    optimizer.setInput0UV(u[0], v[0], stream=stream)
    e_net = optimizer.energy(stream=stream)["total"]
    if e_net <= e_plain:
        return {"used": "network", "energy_network": e_net, "energy_plain": e_plain}
    optimizer.setInput0(u0, stream=stream)
    return {"used": "plain", "energy_network": e_net, "energy_plain": e_plain}


def _case(kw):
    from . import synthetic

    return synthetic.cartesian_case(**kw)


def make_training_set(pdt, torch, n_cases, iters, seed0=1000, C=15, H=640, W=368, roos=True, accel=4,
                      batch=16, workers=None, log=print, steps=DUAL_WEIGHTED_STEPS):
    """(u0, u*, v*) device tensors of n_cases synthetic problems; u* = TGV solution at fixed alpha after
    `iters` iterations from u0 = A^H f with step sizes `steps` (None: the reference's), computed `batch`
    problems at a time. The synthetic cases are generated by a pool of `workers` host processes
    (spawned, so no process inherits a CUDA context) while the GPU solves the previous batch."""
    import concurrent.futures
    import multiprocessing

    Hi = H // 2 if roos else H
    U0 = torch.empty((n_cases, Hi, W), dtype=torch.complex64, device="cuda")
    UT = torch.empty_like(U0)
    VT = torch.empty((n_cases, 2, Hi, W), dtype=torch.complex64, device="cuda")
    kws = [dict(C=C, H=H, W=W, roos=roos, accel=accel, seed=seed0 + i,
                mask_kind="random" if i % 2 == 0 else "regular") for i in range(n_cases)]
    workers = workers or max(1, min(16, (os.cpu_count() or 2) - 1))
    pool = concurrent.futures.ProcessPoolExecutor(workers, mp_context=multiprocessing.get_context("spawn"))
    cases = pool.map(_case, kws, chunksize=1)
    t0 = time.time()
    try:
        _solve_batches(pdt, torch, cases, n_cases, iters, roos, batch, U0, UT, VT, t0, log, steps)
    finally:
        pool.shutdown(cancel_futures=True)
    return U0, UT, VT


def _solve_batches(pdt, torch, cases, n_cases, iters, roos, batch, U0, UT, VT, t0, log, steps):
    for start in range(0, n_cases, batch):
        opts, keep = [], []
        for i in range(start, min(n_cases, start + batch)):
            case = next(cases)
            op = (pdt.mri.MriCartesianRemoveROOSOperator if roos else pdt.mri.MriCartesianOperator)()
            op.setCoilSens(case["sens"])
            op.setMask(case["mask"])
            opt = pdt.mri.TgvMriOptimizer_2c3c()
            prm = opt.getParameters()
            prm.max_iter, prm.reduction, prm.alpha1 = iters - 1, 1.0, case["alpha1"]
            prm.alpha0 = 2 * prm.alpha1
            if steps:
                opt.setSteps(*steps)
            opt.setOperator(op)
            f = torch.from_numpy(case["rawdata"]).cuda()
            opt.setNoisyData(f)
            op.adjoint(f, out=U0[i])
            opt.setInput0(U0[i])
            opts.append((i, opt))
            keep.append((op, f))
        pdt.batch.BatchSolver([o for _, o in opts]).solve()
        for i, opt in opts:
            opt.getResult(out=UT[i])
            opt.getField("vx", out=VT[i, 0])
            opt.getField("vy", out=VT[i, 1])
        torch.cuda.synchronize()
        log(f"targets {min(n_cases, start + batch)}/{n_cases}  {time.time() - t0:.1f}s")


def train(net, U0, UT, VT, epochs=10, batch=8, lr=1e-3, seed=0, log=print):
    """Adam on mini-batches (shuffled per epoch); returns the per-epoch mean losses."""
    rng = np.random.default_rng(seed)
    n = U0.shape[0]
    losses = []
    for ep in range(epochs):
        order = rng.permutation(n)
        tot, cnt = 0.0, 0
        lr_ep = lr * (0.5 ** (ep // max(1, epochs // 3)))
        for s in range(0, n - batch + 1, batch):
            idx = order[s:s + batch].tolist()
            tot += net.train_step(U0[idx].contiguous(), UT[idx].contiguous(), VT[idx].contiguous(), lr=lr_ep)
            cnt += 1
        losses.append(tot / max(cnt, 1))
        log(f"epoch {ep}: loss {losses[-1]:.3e}")
    return losses


def main():
    import torch

    import primaldualtoolbox as pdt

    ap = argparse.ArgumentParser(description="train the warm-start network on engine-generated TGV solutions")
    ap.add_argument("--cases", type=int, default=4096)
    ap.add_argument("--iters", type=int, default=8000, help="dual-weighted iterations per training target")
    ap.add_argument("--shape", default="15,320,320", help="coils,FE,PE of the synthetic problems")
    ap.add_argument("--roos", type=int, default=0, help="1: readout-oversampling removal operator")
    ap.add_argument("--radial", type=int, default=0, help="1: the radial geometry (RADIAL_GEOMETRY) instead")
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--held-out", type=int, default=16)
    ap.add_argument("--out", default=CONFIG4_WEIGHTS)
    args = ap.parse_args()
    C, H, W = (int(x) for x in args.shape.split(","))
    shape = dict(C=C, H=H, W=W, roos=bool(args.roos))
    t0 = time.time()
    if args.radial:
        C, H, W = RADIAL_GEOMETRY["C"], RADIAL_GEOMETRY["N"], RADIAL_GEOMETRY["N"]
        U0, UT, VT = make_radial_training_set(pdt, torch, args.cases, args.iters)
        t_data = time.time() - t0
        H0, HT, HV = make_radial_training_set(pdt, torch, args.held_out, args.iters, seed0=500000)
    else:
        U0, UT, VT = make_training_set(pdt, torch, args.cases, args.iters, **shape)
        t_data = time.time() - t0
        # held-out problems (other seeds) for the report
        H0, HT, HV = make_training_set(pdt, torch, args.held_out, args.iters, seed0=500000, **shape)
    net = WarmStartNet(seed=0)
    t1 = time.time()
    losses = train(net, U0, UT, VT, epochs=args.epochs, batch=args.batch, lr=args.lr)
    torch.cuda.synchronize()
    t_train = time.time() - t1
    held = evaluate(net, torch, H0, HT)
    net.save(args.out, cases=args.cases, target_iters=args.iters, epochs=args.epochs, batch=args.batch, lr=args.lr,
             losses=losses, data_seconds=t_data, train_seconds=t_train, shape=[C, H, W], roos=int(args.roos), accel=4,
             target_steps=None if args.radial else list(DUAL_WEIGHTED_STEPS), radial=int(args.radial), held_out=held)
    print(json.dumps({"out": args.out, "losses": losses, "data_s": round(t_data, 1), "train_s": round(t_train, 1),
                      "held_out": held}))


def evaluate(net, torch, U0, UT):
    """Mean rel-L2 distance to the targets of the network's u and of the plain start u0."""
    n, H, W = U0.shape
    u = torch.empty((1, H, W), dtype=torch.complex64, device=U0.device)
    v = torch.empty((1, 2, H, W), dtype=torch.complex64, device=U0.device)
    e_net, e_plain = [], []
    for i in range(n):
        net.predict(U0[i:i + 1].contiguous(), u, v)
        t = UT[i]
        e_net.append(float(torch.linalg.vector_norm(u[0] - t) / torch.linalg.vector_norm(t)))
        e_plain.append(float(torch.linalg.vector_norm(U0[i] - t) / torch.linalg.vector_norm(t)))
    return {"cases": n, "rel_l2_network": float(np.mean(e_net)), "rel_l2_plain": float(np.mean(e_plain))}


if __name__ == "__main__":
    main()
