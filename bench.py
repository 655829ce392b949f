"""Benchmark: TGV^2 Cartesian MRI reconstruction, 15 coils x 640 x 368 (readout-oversampling removal).

One step = one full TgvMriOptimizer solve of the problem (max_iter = 1000 -> 1001 primal-dual
iterations, the sample's alpha continuation reduction = 2e-8, alpha0 = 2 alpha1) on seeded synthetic
data with the shapes of the reference's knee example (bin/mri_cartesian_test.py).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value  : iterations/s with inputs already resident in HBM (device pointers through the C ABI).
e2e    : iterations/s through the public Python API with pinned host buffers: operator set-up and
         constant upload, setNoisyData (H2D), solve, getResult (D2H) inside every timed step.
--impl reference : the reference algorithm on the host cores (the CPU oracle restatement, all
         threads), a bounded sample of the same workload per step.
Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "primal-dual-toolbox_gb300")
for _p in (PKG_DIR, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

C, H, W = 15, 640, 368
MAX_ITER = 1000
ITERS = MAX_ITER + 1
REDUCTION = 2e-8
METRIC = "TGV MRI 15c 640x368: iters/s and time to 1e-4 rel err, warm-start vs plain"
WORKLOAD = "tgv2_cartesian_roos_15c_640x368_1001it"
L2_FLUSH_BYTES = 256 << 20


def _rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(value, dist=None):
    """Maximum of a per-rank float over all ranks (identity without a process group). Replicas only: the
    data path has no collective; this is the timing barrier's max-over-ranks."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(iters_per_step, steps, world, t_max):
    """Whole-job iterations/s: every rank solves its own reconstruction (weak scaling)."""
    return iters_per_step * steps * world / t_max


def _synthetic():
    """The seeded phantom generator (primaldualtoolbox/synthetic.py, numpy only), loaded from its file
    without importing the package: the reference arm must not load libpdt.so."""
    import importlib.util

    name = "pdt_bench_synthetic"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, os.path.join(PKG_DIR, "primaldualtoolbox", "synthetic.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        sys.modules[name] = mod
    return sys.modules[name]


def _problem(seed=0):
    return _synthetic().cartesian_case(C=C, H=H, W=W, roos=True, seed=seed)


def _config(case, world):
    """The workload description both arms print."""
    ns = int((case["mask"] != 0).any(axis=0).sum())
    return {"workload": WORKLOAD, "coils": C, "fe": H, "pe": W, "image": [H // 2, W],
            "iterations_per_step": ITERS, "reduction": REDUCTION, "sampled_pe_lines": ns,
            "accel": round(W / ns, 2), "l2": "flushed between steps (256 MB write)",
            "parallelism": f"replicas{world}"}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["bf16_tflops"])
    except Exception:
        return 1900.0


def _ncu_traffic():
    """Per-launch DRAM bytes of each kernel from the committed ncu summary (profiles/dram_traffic.txt)."""
    out = {}
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if os.path.exists(path):
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and not line.startswith("#"):
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def _phase_bytes_case(C, Hf, W, ns, G, roos):
    """Algorithmic bytes of one iteration of a Cartesian TGV-MRI problem under the engine's layout
    (sampled columns only; each logical array read or written once), per kernel phase."""
    Hi = Hf // 2 if roos else Hf
    N = Hi * W
    c8 = 8
    return {
        "cart_rows_fwd": c8 * (N + C * N + C * ns * Hi),
        "cart_cols_prox": c8 * (C * ns * Hi + 3 * C * ns * Hf + C * ns * Hi) + 4 * ns * Hf,
        "cart_rows_adj": c8 * (C * ns * Hi + C * N + G * N),
        "mri_dual_tgv": c8 * N * (8 + 5),
        "mri_primal_tgv": c8 * N * (8 + G + 6),
    }


def _phase_bytes(ns, G, fused_dual=False):
    """Algorithmic bytes per launch of each kernel phase (each logical array read or written once). With
    the dual update run by extra blocks of the adjoint-rows launch (fused_dual), that launch moves both."""
    Hi = H // 2
    c8 = 8
    out = {
        # ubar + sens rows in, t1 (sampled columns) out
        "cart_rows_fwd": c8 * (Hi * W + C * Hi * W + C * ns * Hi),
        # t1, f, r in; r, t2 out; mask of sampled columns
        "cart_cols_prox": c8 * (C * ns * Hi + 3 * C * ns * H + C * ns * Hi) + 4 * ns * H,
        # t2 + sens rows in, K^H r partial sums out
        "cart_rows_adj": c8 * (C * ns * Hi + C * Hi * W + G * Hi * W),
        # dual: ub, vb(2), p(2), q(3) in; p(2), q(3) out
        "mri_dual_tgv": c8 * Hi * W * (8 + 5),
        # primal: u, v(2), p(2), q(3), G K^H r partials in; u, ub, v(2), vb(2) out
        "mri_primal_tgv": c8 * Hi * W * (8 + G + 6),
    }
    if fused_dual:
        out["cart_rows_adj"] += out.pop("mri_dual_tgv")
    return out


def run_ours(args):
    import torch

    import primaldualtoolbox as pdt

    rank, world, local = _rank_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    case = _problem(seed=rank)
    ns = int((case["mask"] != 0).any(axis=0).sum())
    dev = {k: torch.from_numpy(np.ascontiguousarray(case[k])).cuda() for k in ("rawdata", "sens", "mask")}
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    op = pdt.mri.MriCartesianRemoveROOSOperator()
    op.setCoilSens(dev["sens"])
    op.setMask(dev["mask"])
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.max_iter, prm.reduction, prm.alpha1 = MAX_ITER, REDUCTION, case["alpha1"]
    prm.alpha0 = 2 * prm.alpha1
    opt.setOperator(op)
    u0 = torch.empty((H // 2, W), dtype=torch.complex64, device="cuda")
    op.adjoint(dev["rawdata"], out=u0, stream=stream)

    def step():
        # one fresh solve as the reference's solve() runs it on a new optimizer: r = 0, u = ubar = A^H f
        # (computed inside the step, tgvmrioptimizer.cu:112-118), v = p = q = 0
        flush.zero_()  # evict L2 between steps (inputs ~120 MB < 129 MB L2)
        opt.setNoisyData(dev["rawdata"], stream=stream)
        op.adjoint(dev["rawdata"], out=u0, stream=stream)
        opt.setInput0(u0, stream=stream)
        opt.solve(stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    n0 = pdt.launch_count()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = pdt.launch_count() - n0
    dev_s = ev0.elapsed_time(ev1) / 1e3
    parity = _parity_fp64(case, opt.getResult()) if rank == 0 else None
    t_max = max_over_ranks(dev_s, dist)
    value = replica_throughput(ITERS, args.steps, world, t_max)

    # per-kernel timing (CUDA events on the launching stream) for the roofline of the dominant kernel
    phases = opt.profile(iters=50, stream=stream)
    G = _khr_planes(op.tuning())
    fused_dual = "solver_dual=adjoint_launch" in op.tuning()
    bytes_per = _phase_bytes(ns, G, fused_dual)
    per_iter_ms = sum(phases.values())
    dom = max(phases, key=phases.get)
    hbm, src = _peaks()
    traffic = _ncu_traffic()
    achieved = bytes_per.get(dom, 0) / (phases[dom] / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": hbm, "peak_source": src,
            "unit": "GB/s", "frac": round(achieved / hbm, 4),
            "traffic": traffic.get(dom + "+dual" if fused_dual and dom == "cart_rows_adj" else dom),
            "algorithmic_bytes": bytes_per.get(dom), "launch_ms": round(phases[dom], 5),
            "share": round(phases[dom] / per_iter_ms, 3)}
    if fused_dual and dom == "cart_rows_adj":
        roof["launch_includes"] = "the solver's dual update (extra blocks on the SMs the row tiles leave free)"
    phase_info = {k: {"ms": round(v, 5), "GB/s": round(bytes_per.get(k, 0) / (v / 1e3) / 1e9, 1)}
                  for k, v in phases.items()}
    tuning = op.tuning()
    if "rows_adj=tensor_dft" in tuning and "cart_rows_adj" in phases:
        # tensor-core DFT adjoint rows: one real GEMM pass is 2 (C Hi) (2 W) (2 ns) flops; the TF32 hi/lo
        # split executes three; the TF32 peak is half the measured dense BF16 rate (the tensor cores'
        # TF32 : BF16 ratio)
        flop = 3 * 2 * (C * (H // 2)) * (2 * W) * (2 * ns)
        tf32_peak = _bf16_peak() / 2
        ach = flop / (phases["cart_rows_adj"] / 1e3) / 1e12
        phase_info["cart_rows_adj"]["tensor"] = {
            "bound": "tensor", "achieved": round(ach, 1), "peak": round(tf32_peak, 1), "unit": "TFLOP/s",
            "frac": round(ach / tf32_peak, 4), "flop_executed": flop, "dtype": "tf32x3 (FP32 accuracy)",
            "peak_source": "measured bf16 / 2"}

    cufft = run_cufft(pdt, torch, case, dev, op, phases) if args.cufft else None

    conv = None
    if args.accuracy:
        from primaldualtoolbox import warmstart

        conv = {"tgv_mri_15c_640x368_roos": _cartesian_convergence(
            pdt, torch, case, stream, True, per_iter_s=t_max / args.steps / ITERS, weights=warmstart.DEFAULT_WEIGHTS,
            max_plain=200000)}
        conv["config4_15c_320x320"] = _cartesian_convergence(pdt, torch, _synthetic().cartesian_case(seed=4000, **CFG4),
                                                             stream, False, weights=warmstart.CONFIG4_WEIGHTS)

    # e2e: the public API with pinned host buffers, every input uploaded and the result read back
    host = {k: pdt.pinned_empty(case[k].shape, case[k].dtype) for k in ("rawdata", "sens", "mask")}
    for k in host:
        host[k][...] = case[k]
    h2d = sum(host[k].nbytes for k in host)
    d2h = (H // 2) * W * 8

    def e2e_step():
        flush.zero_()
        o = pdt.mri.MriCartesianRemoveROOSOperator()
        o.setCoilSens(host["sens"])
        o.setMask(host["mask"])
        s = pdt.mri.TgvMriOptimizer_2c3c()
        p = s.getParameters()
        p.max_iter, p.reduction, p.alpha1 = MAX_ITER, REDUCTION, case["alpha1"]
        p.alpha0 = 2 * p.alpha1
        s.setOperator(o)
        s.setNoisyData(host["rawdata"])
        s.solve()
        return s.getResult()

    e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e_val = replica_throughput(ITERS, e_steps, world, e2e_s)

    # e2e through the streaming pipeline: slices arrive as host arrays and leave as host images, uploads
    # and downloads overlapping the solves (reused operators and optimizers, two slots)
    streamed = None
    if args.stream_slices > 0:
        from primaldualtoolbox import pipeline

        distinct = [case] + [_problem(seed=1000 * (rank + 1) + j) for j in range(3)]
        slices = [distinct[j % len(distinct)] for j in range(args.stream_slices)]
        ss = pipeline.SliceStream(C, H, W, roos=True, alpha1=case["alpha1"], reduction=REDUCTION, max_iter=MAX_ITER,
                                  torch=torch)
        for _ in ss.run(distinct[:2]):  # warm-up: operators, tuning, graphs
            pass
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        n_done = sum(1 for _ in ss.run(slices))
        st_s = max_over_ranks(time.perf_counter() - t0, dist)
        streamed = {"value": round(replica_throughput(ITERS, n_done, world, st_s), 1), "unit": "iters/s",
                    "slices": n_done, "slices_per_s": round(n_done * world / st_s, 3),
                    "h2d_bytes_per_slice": int(2 * C * H * W * 8), "d2h_bytes_per_slice": int((H // 2) * W * 8),
                    "note": "host rawdata + coil maps in, host image out; same mask for all slices"}

    denoising = run_denoising(pdt, torch) if args.denoising else None
    if denoising is not None:
        denoising["hbm_resident"] = run_denoising_hbm(pdt, torch)

    radial = None
    if args.radial_slices > 0:
        radial = run_radial(pdt, torch, args.radial_slices, args.radial_iters, converge=bool(args.accuracy))

    batched = None
    if args.batch_cases > 0:
        batched = run_batched(pdt, torch, args.batch_cases, args.batch_iters, steps=2, warmup=1)

    line = None
    if rank == 0:
        cpu = _cpu_baseline(case, seconds=args.cpu_seconds)
        c2 = conv["tgv_mri_15c_640x368_roos"] if conv else None
        if c2 and c2["plain"]["iterations"]:
            # the host path needs the same iteration count (the FP32 mirror follows the same iterates)
            cpu["time_to_1e-4_s_plain"] = round(c2["plain"]["iterations"] / cpu["value"], 1)
        line = {
            "metric": METRIC, "value": round(value, 1), "unit": "iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_max / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": _config(case, world),
            "e2e": {"value": round(e2e_val, 1), "unit": "iters/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e_steps},
            "gpu_launches": int(launches),
            "roofline": roof,
            "phases": phase_info,
            "tuning": tuning,
            "cpu_baseline": cpu,
            "parity": parity,
            "time_to_1e-4": conv,
            "e2e_streamed": streamed,
            "batched": batched,
            "radial": radial,
            "denoising": denoising,
            "beside_cufft": cufft,
            "clocks": clk.summary(),
            "wall_s": round(wall, 3),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return line


REF_SAMPLE_ITERS = 24  # iterations per step of the --impl reference arm (about 1.6 s on 16 host cores)
STAR_ITERS = 60000      # dual-weighted iterations for the converged solution u*
CFG4 = dict(C=15, H=320, W=320, roos=False, accel=4)  # the learned-warm-start configuration


def _fixed_alpha_optimizer(pdt, case, dev, stream, roos):
    op = (pdt.mri.MriCartesianRemoveROOSOperator if roos else pdt.mri.MriCartesianOperator)()
    op.setCoilSens(dev["sens"])
    op.setMask(dev["mask"])
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.reduction, prm.alpha1 = 1.0, case["alpha1"]
    prm.alpha0 = 2 * prm.alpha1
    opt.setOperator(op)
    opt.setNoisyData(dev["rawdata"], stream=stream)
    return op, opt, prm


def _iterations_to(pdt, torch, opt, prm, u_star, n_star, stream, target, chunk, max_iters):
    """Runs `opt` in chunks of `chunk` iterations until rel-L2 to u_star <= target (FP64 GPU reduction
    between chunks); returns (iterations, final error)."""
    u = torch.empty_like(u_star)
    prm.max_iter = chunk - 1
    it, err = 0, None
    while it < max_iters:
        opt.solve(stream=stream)
        it += chunk
        opt.getResult(out=u, stream=stream)
        torch.cuda.synchronize()
        err = pdt.dist2(u, u_star) ** 0.5 / n_star
        if err <= target:
            break
    return (it if err is not None and err <= target else None), err


def _per_iteration_s(opt, prm, torch, stream, n=2000):
    prm.max_iter = n - 1
    opt.solve(stream=stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    opt.solve(stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / n


def time_to_accuracy(pdt, torch, make, u0, stream, per_iter_s=None, weights=None, steps=None, target=1e-4,
                     max_plain=400000, max_dual=60000):
    """Wall time for a fixed-alpha TGV-MRI iteration (reduction 1) to reach rel-L2 <= target to its
    converged solution u*, four ways: the reference's step sizes from the plain start u0 = A^H f (`plain`),
    the same from the learned warm start (`warm_start`: the network's (u, v), kept only when its FP64
    energy is lower), and both starts with the dual-weighted step sizes (`dual_weighted`,
    `warm_start_dual_weighted`: sigma / tau = 1024 instead of 2, tau sigma (12 + |K|^2) = 0.8). All four
    converge to the same saddle point. `make()` returns a fresh (operator, optimizer, parameters) with the
    data set; u0 is the device image A^H f. u* is the engine's dual-weighted iterate after STAR_ITERS
    iterations; its change over 2000 further iterations with the reference's steps is reported. Times are
    iterations x the timed per-iteration cost (+ the network's inference and energy check); errors are
    FP64 GPU reductions."""
    from primaldualtoolbox import warmstart

    op, ref, prm = make()
    if steps is None:
        steps = warmstart.dual_weighted_steps(op.norm(iters=40))
    if per_iter_s is None:
        per_iter_s = _per_iteration_s(ref, prm, torch, stream)
        op, ref, prm = make()
    ref.setSteps(*steps)
    prm.max_iter = STAR_ITERS - 1
    ref.solve(stream=stream)
    shape = tuple(u0.shape)
    u_star = torch.empty(shape, dtype=torch.complex64, device="cuda")
    ref.getResult(out=u_star, stream=stream)
    ref.setSteps(0, 0)
    prm.max_iter = 1999
    ref.solve(stream=stream)
    u_ref = torch.empty_like(u_star)
    ref.getResult(out=u_ref, stream=stream)
    torch.cuda.synchronize()
    n_star = pdt.dist2(u_star) ** 0.5
    stationarity = pdt.dist2(u_ref, u_star) ** 0.5 / n_star
    del ref
    out = {"target_rel_l2": target, "alpha": "fixed (reduction 1)", "per_iteration_ms": round(per_iter_s * 1e3, 5),
           "u_star": {"iterations": STAR_ITERS, "steps": "dual_weighted",
                      "change_over_2000_reference_iterations": stationarity},
           "dual_weighted_steps": {"tau": steps[0], "sigma": steps[1]},
           "start_rel_l2_plain": pdt.dist2(u0, u_star) ** 0.5 / n_star}

    net, inf_ms = None, 0.0
    if weights and os.path.exists(weights):
        net = warmstart.WarmStartNet(weights=weights)
        uw = torch.empty((1,) + shape, dtype=torch.complex64, device="cuda")
        vw = torch.empty((1, 2) + shape, dtype=torch.complex64, device="cuda")
        net.predict(u0.reshape((1,) + shape), uw, vw, stream=stream)  # warm-up
        _, o, _ = make()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        choice = warmstart.warm_start(o, net, u0, torch, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        inf_ms = e0.elapsed_time(e1)
        out["warm_start_choice"] = {k: (round(v, 6) if isinstance(v, float) else v) for k, v in choice.items()}
        out["warm_start_choice"]["inference_and_energy_ms"] = round(inf_ms, 3)
        ws = torch.empty_like(u_star)
        o.getResult(out=ws, stream=stream)
        torch.cuda.synchronize()
        out["warm_start_choice"]["start_rel_l2"] = pdt.dist2(ws, u_star) ** 0.5 / n_star
        out["weights"] = os.path.relpath(weights, ROOT)

    def leg(name, learned, dual):
        _, o, p = make()
        if learned:
            warmstart.warm_start(o, net, u0, torch, stream=stream)
        else:
            o.setInput0(u0, stream=stream)
        if dual:
            o.setSteps(*steps)
        cap = max_dual if dual else max_plain
        it, err = _iterations_to(pdt, torch, o, p, u_star, n_star, stream, target, 250 if dual else 1000, cap)
        res = {"iterations": it, "final_rel_l2": err}
        if it:
            res["ms"] = round(it * per_iter_s * 1e3 + (inf_ms if learned else 0.0), 3)
        else:
            res["not_reached_within"] = cap
        out[name] = res

    leg("plain", False, False)
    leg("dual_weighted", False, True)
    if net is not None:
        leg("warm_start", True, False)
        leg("warm_start_dual_weighted", True, True)
    base = out["plain"].get("ms") or max_plain * per_iter_s * 1e3  # a lower bound when not reached
    for k in ("dual_weighted", "warm_start", "warm_start_dual_weighted"):
        if k in out and out[k].get("ms"):
            out[k]["speedup_vs_plain"] = round(base / out[k]["ms"], 2)
            if not out["plain"].get("ms"):
                out[k]["speedup_is_lower_bound"] = True
    return out


def _cartesian_convergence(pdt, torch, case, stream, roos, **kw):
    dev = {k: torch.from_numpy(np.ascontiguousarray(case[k])).cuda() for k in ("rawdata", "sens", "mask")}

    def make():
        return _fixed_alpha_optimizer(pdt, case, dev, stream, roos)

    op, _, _ = make()
    Hf, Wd = case["mask"].shape
    u0 = torch.empty((Hf // 2 if roos else Hf, Wd), dtype=torch.complex64, device="cuda")
    op.adjoint(dev["rawdata"], out=u0, stream=stream)
    torch.cuda.synchronize()
    return time_to_accuracy(pdt, torch, make, u0, stream, **kw)


def _khr_planes(tuning):
    """K^H r planes the adjoint row phase writes and the image step reads: 1 when the coil groups are
    reduced in a thread-block cluster, else one partial image per coil group (from the operator's
    tuning report, e.g. '... rows_adj=register_fft(warps=4,coil_groups=6,partials) ...')."""
    import re

    m = re.search(r"coil_groups=(\d+)(,cluster|,partials)?", tuning)
    if not m:
        return 1
    return 1 if m.group(2) == ",cluster" else int(m.group(1))


def _batch_khr_planes(tuning):
    """(K^H r planes, lane-FFT rows) of an operator inside a batch: its `in_batch=lane_fft_rows(
    batch_adj_groups=G,partials|cluster)` report where it has lane-FFT rows (a batch runs those, with at
    most two coil groups), else the solo figures."""
    m = re.search(r"batch_adj_groups=(\d+)(,cluster|,partials)", tuning)
    if not m:
        return _khr_planes(tuning), False
    return (1 if m.group(2) == ",cluster" else int(m.group(1))), True


FP64_FIXTURE = os.path.join(ROOT, "tests", "golden", "config2_fp64.npz")


def _parity_fp64(case, u):
    """rel-L2 of the timed solve's result to the FP64 CPU oracle's result of the same 1001 iterations on the
    same inputs (tests/golden/config2_fp64.npz, written by tests/golden/make_config2_fp64.py)."""
    import hashlib

    if not os.path.exists(FP64_FIXTURE):
        return {"unavailable": "tests/golden/config2_fp64.npz is missing"}
    z = np.load(FP64_FIXTURE)
    h = hashlib.sha256()
    for k in ("rawdata", "sens", "mask"):
        h.update(np.ascontiguousarray(case[k]).tobytes())
    ref = z["u"].astype(np.complex128)
    err = float(np.linalg.norm(u.astype(np.complex128) - ref) / np.linalg.norm(ref))
    return {"rel_l2_fp64": err, "tolerance": 1e-4, "pass": bool(err <= 1e-4),
            "oracle": f"FP64 CPU oracle, the same {int(z['max_iter']) + 1} iterations from the same inputs "
                      f"(tests/golden/config2_fp64.npz: {float(z['seconds']):.0f} s on {int(z['threads'])} threads)",
            "inputs_identical_to_oracle_run": h.hexdigest() == str(z["inputs_sha256"])}


def _cpu_baseline(case, seconds=10.0, threads=None):
    """The reference iteration on the host cores: the CPU oracle restatement (FP32 mirror), all threads."""
    from oracle import oracle

    threads = threads or os.cpu_count()
    oracle.set_threads(threads)
    u0 = oracle.op_apply("cartesian_roos", case["sens"], case["mask"], case["rawdata"], adjoint=True, prec=32)

    def run(n):
        t0 = time.perf_counter()
        oracle.op_solve("cartesian_roos", case["sens"], case["mask"], case["rawdata"], "tgv_mri",
                        alpha0=case["alpha0"], alpha1=case["alpha1"], reduction=REDUCTION, max_iter=n - 1, u0=u0,
                        prec=32)
        return time.perf_counter() - t0

    n = max(2, int(seconds / max(run(2) / 2, 1e-3)))
    dt = run(n)
    # the FP64 oracle of the same iteration (the precision the parity figure is measured against)
    t0 = time.perf_counter()
    n64 = max(2, n // 3)
    oracle.op_solve("cartesian_roos", case["sens"], case["mask"], case["rawdata"], "tgv_mri", alpha0=case["alpha0"],
                    alpha1=case["alpha1"], reduction=REDUCTION, max_iter=n64 - 1, u0=u0.astype(np.complex128),
                    prec=64)
    fp64 = {"value": round(n64 / (time.perf_counter() - t0), 3), "unit": "iters/s", "iterations": n64}
    return {"value": round(n / dt, 3), "unit": "iters/s", "cores": threads, "kind": "port", "fp64": fp64,
            "sample": f"the first {n} of the {ITERS} iterations of one solve from u0 = A^H f (the one-off A^H f, "
                      f"about one iteration's operator work, outside the sample), FP32 mirror of the reference "
                      f"iteration"}


BATCH_SIZES = [(192, 192), (256, 256), (320, 320), (640, 368)]


def _batch_specs(n, seed0=3000):
    """Config-3 style batch: sizes from BATCH_SIZES, coils U{8..32}, acceleration U{2..8}, regular or
    random phase-encode masks, plain (no ROOS) Cartesian operators, one seed per case."""
    rng = np.random.default_rng(seed0)
    out = []
    for i in range(n):
        Hf, Wd = BATCH_SIZES[int(rng.integers(len(BATCH_SIZES)))]
        out.append(dict(C=int(rng.integers(8, 33)), H=Hf, W=Wd, roos=False, accel=int(rng.integers(2, 9)),
                        mask_kind="regular" if rng.random() < 0.5 else "random", seed=seed0 + i))
    return out


def run_batched(pdt, torch, n_cases, iters, steps, warmup):
    """n_cases independent TGV-MRI reconstructions solved together (primaldualtoolbox.batch, one CUDA
    graph per 10 iterations). Returns problem-iterations/s and the whole-iteration HBM roofline: the
    working set (several GB) is far larger than L2, so the bytes come from HBM."""
    import concurrent.futures
    import multiprocessing

    from primaldualtoolbox import warmstart

    specs = _batch_specs(n_cases)
    t0 = time.perf_counter()
    with concurrent.futures.ProcessPoolExecutor(max(1, min(16, (os.cpu_count() or 2) - 1)),
                                                mp_context=multiprocessing.get_context("spawn")) as pool:
        cases = list(pool.map(warmstart._case, specs, chunksize=1))
    t_gen = time.perf_counter() - t0
    opts, ops, nbytes, pix, adj_rows = [], [], 0, 0, {}
    for spec, case in zip(specs, cases):
        op = pdt.mri.MriCartesianOperator()
        op.setCoilSens(case["sens"])
        op.setMask(case["mask"])
        opt = pdt.mri.TgvMriOptimizer_2c3c()
        prm = opt.getParameters()
        prm.max_iter, prm.reduction, prm.alpha1 = iters - 1, REDUCTION, case["alpha1"]
        prm.alpha0 = 2 * prm.alpha1
        opt.setOperator(op)
        opt.setNoisyData(case["rawdata"])
        ns = int((case["mask"] != 0).any(axis=0).sum())
        tuning = op.tuning()
        G, lane_in_batch = _batch_khr_planes(tuning)
        adj = "tensor_dft" if "rows_adj=tensor_dft" in tuning and not lane_in_batch else "lane_fft"
        adj_rows[adj] = adj_rows.get(adj, 0) + 1
        nbytes += sum(_phase_bytes_case(spec["C"], spec["H"], spec["W"], ns, G, False).values())
        pix += spec["H"] * spec["W"]
        opts.append(opt)
        ops.append(op)
    del cases
    batch = pdt.batch.BatchSolver(opts)
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        batch.solve(stream=stream)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        batch.solve(stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    dt = ev0.elapsed_time(ev1) / 1e3
    hbm, src = _peaks()
    achieved = nbytes * iters * steps / dt / 1e9
    return {"workload": f"batch_{n_cases}_cartesian_tgv2_mixed", "cases": n_cases, "iterations_per_case": iters,
            "sizes": [f"{a}x{b}" for a, b in BATCH_SIZES], "coils": "U{8..32}", "accel": "U{2..8}",
            "steps": steps, "warmup": warmup, "value": round(n_cases * iters * steps / dt, 1),
            "unit": "problem-iterations/s", "ms_per_step": round(dt / steps * 1e3, 3),
            "pixel_iterations_per_s": round(pix * iters * steps / dt, 1),
            "roofline": {"bound": "hbm", "kernel": "whole iteration (all phases)", "achieved": round(achieved, 1),
                         "peak": hbm, "peak_source": src, "unit": "GB/s", "frac": round(achieved / hbm, 4),
                         "algorithmic_bytes_per_iteration_all_cases": int(nbytes)},
            "adjoint_rows_chosen": adj_rows, "case_generation_s": round(t_gen, 1)}


RAD_N, RAD_C, RAD_SPOKES, RAD_RO, RAD_OSF, RAD_KW = 256, 12, 64, 512, 1.5, 3


def _radial_problem(pdt, seed):
    """Config 5: 256 x 256 image, 12 coils, 64 golden-angle spokes x 512 readout samples (2x readout
    oversampling), Kaiser-Bessel width 3 on a 1.5x grid, density weights sqrt|k|, a seeded phantom and
    seeded coil maps; f = A u + 1 % complex noise (primaldualtoolbox.warmstart.radial_problem)."""
    from primaldualtoolbox import warmstart

    return warmstart.radial_problem(pdt, seed, N=RAD_N, C=RAD_C, spokes=RAD_SPOKES, readout=RAD_RO, osf=RAD_OSF,
                                    kernel_width=RAD_KW)


def _radial_bytes():
    """Algorithmic bytes of one radial TGV-MRI iteration, each array pass counted once: image x coil maps
    in and out, the padded row transforms and the oversampled grid written and read in both directions,
    the samples' dual r (read, write), data and weights, and the image side (dual 13 + primal 15 planes)."""
    G = int(np.ceil(RAD_OSF * RAD_N))
    Ns = RAD_SPOKES * RAD_RO
    c8 = 8
    fwd = c8 * (RAD_N * RAD_N * (1 + RAD_C) + 2 * RAD_C * RAD_N * G + 2 * RAD_C * G * G)
    prox = c8 * RAD_C * Ns * 4 + 4 * Ns
    adj = c8 * (2 * RAD_C * G * G + 2 * RAD_C * RAD_N * G + RAD_N * RAD_N * (RAD_C + 1))
    return fwd + prox + adj + c8 * RAD_N * RAD_N * 28


def run_radial(pdt, torch, slices, iters, converge=True):
    """Config 5: one radial slice alone, and `slices` slices advanced together (BatchSolver)."""
    probs = [_radial_problem(pdt, seed=s) for s in range(slices)]
    opts = []
    for op, f, a1 in probs:
        opt = pdt.mri.TgvMriOptimizer_2c2c()
        prm = opt.getParameters()
        prm.max_iter, prm.reduction, prm.alpha1 = iters - 1, 2.0 ** -8, a1
        prm.alpha0 = 2 * a1
        opt.setOperator(op)
        opt.setNoisyData(f)
        opts.append(opt)
    stream = torch.cuda.current_stream()
    hbm, src = _peaks()
    nbytes = _radial_bytes()

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    t1 = timed(lambda: opts[0].solve(stream=stream), 3)
    batch = pdt.batch.BatchSolver(opts)
    tb = timed(lambda: batch.solve(stream=stream), 2)
    conv = None
    if converge:
        # time to rel-L2 1e-4 of one slice: reference vs dual-weighted steps, plain vs learned start
        from primaldualtoolbox import warmstart

        op0, f0, a10 = probs[0]
        fd = torch.from_numpy(np.ascontiguousarray(f0)).cuda()

        def make():
            o = pdt.mri.TgvMriOptimizer_2c2c()
            p = o.getParameters()
            p.reduction, p.alpha1, p.alpha0 = 1.0, a10, 2 * a10
            o.setOperator(op0)
            o.setNoisyData(fd, stream=stream)
            return op0, o, p

        u0 = torch.empty((RAD_N, RAD_N), dtype=torch.complex64, device="cuda")
        op0.adjoint(fd, out=u0, stream=stream)
        torch.cuda.synchronize()
        conv = time_to_accuracy(pdt, torch, make, u0, stream, weights=warmstart.RADIAL_WEIGHTS, max_plain=150000)
        conv["operator_norm"] = op0.norm(iters=40)
    return {"workload": f"radial_tgv2_{RAD_C}c_{RAD_N}x{RAD_N}_{RAD_SPOKES}spokes_x{RAD_RO}",
            "osf": RAD_OSF, "kernel_width": RAD_KW, "iterations_per_slice": iters, "tuning": probs[0][0].tuning(),
            "single_slice": {"value": round(iters / t1, 1), "unit": "iters/s"},
            "batched": {"slices": slices, "value": round(slices * iters / tb, 1), "unit": "slice-iterations/s",
                        "roofline": {"bound": "hbm", "kernel": "whole iteration (all phases)",
                                     "achieved": round(nbytes * slices * iters / tb / 1e9, 1), "peak": hbm,
                                     "peak_source": src, "unit": "GB/s",
                                     "frac": round(nbytes * slices * iters / tb / 1e9 / hbm, 4),
                                     "algorithmic_bytes_per_slice_iteration": int(nbytes)}},
            "time_to_1e-4": conv}


def run_denoising(pdt, torch, reps=3):
    """Config 1 (TvOptimizer, 512 x 512 float32, lambda 10, 500 -> 501 iterations) and the same image
    through TgvOptimizer (alpha1 0.1, alpha0 0.2), data resident. Algorithmic bytes per iteration of the
    fused kernels: TV reads u-bar, p (2), u, f and writes p (2), u, u-bar = 9 planes (+ 2 halo re-reads
    not counted); TGV 12 reads + 11 writes of the 11-plane state (f included) = 23 planes."""
    from primaldualtoolbox import synthetic

    f = torch.from_numpy(synthetic.tv_phantom(512, 512, seed=0)[0]).cuda()  # the noisy image
    stream = torch.cuda.current_stream()
    hbm, src = _peaks()
    out = {}
    for name, cls, planes in (("tv_rof", pdt.denoising.TvOptimizer_2f, 9), ("tgv", pdt.denoising.TgvOptimizer_2f, 23)):
        opt = cls()
        prm = opt.getParameters()
        prm.max_iter, prm.Lambda = 500, 10.0
        if name == "tgv":
            prm.alpha1, prm.alpha0 = 0.1, 0.2
        opt.setNoisyData(f, stream=stream)
        opt.solve(stream=stream)  # warm-up: state and graph
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            opt.solve(stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        dt = e0.elapsed_time(e1) / 1e3 / reps
        nbytes = 4 * 512 * 512 * planes
        out[name] = {"value": round(501 / dt, 1), "unit": "iters/s", "ms_per_solve": round(dt * 1e3, 3),
                     "roofline": {"bound": "hbm", "achieved": round(nbytes * 501 / dt / 1e9, 1), "peak": hbm,
                                  "peak_source": src, "unit": "GB/s",
                                  "frac": round(nbytes * 501 / dt / 1e9 / hbm, 4),
                                  "algorithmic_bytes_per_iteration": nbytes,
                                  "note": "4 MB state stays in L2 within a solve"}}
    out["workload"] = "denoise_512x512_f32_501it"
    return out


def run_denoising_hbm(pdt, torch, reps=3, iters=21):
    """The fused primal-dual step kernels on HBM-resident images (the 512 x 512 benchmark image's state
    fits in L2): TV and TGV on an 8192 x 8192 float32 image (TGV state 2 x 11 planes = 5.6 GB) and TGV on a
    complex 8192 x 4096 image, each a seeded phantom tiled to size, `iters` iterations per solve. Bytes per
    iteration as run_denoising (TV 9 planes, TGV 23 planes of the pixel type)."""
    from primaldualtoolbox import synthetic

    base = synthetic.tv_phantom(512, 512, seed=0)[0].astype(np.float32)
    stream = torch.cuda.current_stream()
    hbm, src = _peaks()
    out = {}
    cases = (("tv_rof_8192x8192_f32", pdt.denoising.TvOptimizer_2f, 9, (8192, 8192), False),
             ("tgv_8192x8192_f32", pdt.denoising.TgvOptimizer_2f, 23, (8192, 8192), False),
             ("tgv_8192x4096_c64", pdt.denoising.TgvOptimizer_2c, 23, (8192, 4096), True))
    for name, cls, planes, (Hh, Ww), cplx in cases:
        img = np.tile(base, (Hh // 512, Ww // 512))
        if cplx:
            img = (img * np.exp(1j * np.linspace(0, 3, Ww))[None, :]).astype(np.complex64)
        f = torch.from_numpy(img).cuda()
        opt = cls()
        prm = opt.getParameters()
        prm.max_iter, prm.Lambda = iters - 1, 10.0
        if "tgv" in name:
            prm.alpha1, prm.alpha0 = 0.1, 0.2
        opt.setNoisyData(f, stream=stream)
        opt.solve(stream=stream)  # warm-up: state and graph
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            opt.solve(stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        dt = e0.elapsed_time(e1) / 1e3 / reps / iters
        nbytes = (8 if cplx else 4) * Hh * Ww * planes
        out[name] = {"ms_per_iteration": round(dt * 1e3, 4),
                     "roofline": {"bound": "hbm", "achieved": round(nbytes / dt / 1e9, 1), "peak": hbm,
                                  "peak_source": src, "unit": "GB/s", "frac": round(nbytes / dt / 1e9 / hbm, 4),
                                  "algorithmic_bytes_per_iteration": nbytes}}
        del opt, f
    out["note"] = ("TV runs four iterations per launch (temporal blocking in shared memory), so its bytes per "
                   "iteration are the algorithmic ones of one iteration while the kernel passes over the state once "
                   "per four")
    return out


def run_cufft(pdt, torch, case, dev, op, phases, reps=50):
    """The Cartesian operator (config 2: 15 coils x 640 x 368, ROOS) timed beside cuFFT: the fused
    hand-written kernels of libpdt.so against the reference's launch chain on torch.fft (shifts, batched
    fft2/ifft2, mask, conj-sens combine, pad/crop), same device inputs, CUDA events, warm L2. Also the
    batched cuFFT fft2 alone (the library transform without any of the operator's other passes) and one
    operator half of a solver iteration (k-space prox + adjoint) against the solver's fused phases."""
    from primaldualtoolbox.cufft_companion import CartesianCufft

    stream = torch.cuda.current_stream()
    ref = CartesianCufft(dev["sens"], dev["mask"], True, torch)
    u = torch.empty((H // 2, W), dtype=torch.complex64, device="cuda")
    op.adjoint(dev["rawdata"], out=u, stream=stream)
    k = torch.empty((C, H, W), dtype=torch.complex64, device="cuda")
    r = torch.zeros_like(k)

    def timed(fn):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    t = {
        "ours_forward_ms": timed(lambda: op.forward(u, out=k, stream=stream)),
        "ours_adjoint_ms": timed(lambda: op.adjoint(dev["rawdata"], out=u, stream=stream)),
        "cufft_forward_ms": timed(lambda: ref.forward(u)),
        "cufft_adjoint_ms": timed(lambda: ref.adjoint(dev["rawdata"])),
        "cufft_fft2_only_ms": timed(lambda: torch.fft.fft2(k, norm="ortho")),
        "cufft_iteration_operator_ms": timed(lambda: ref.prox_step(u, r, dev["rawdata"], 0.125, 1.0)),
    }
    ours_iter = sum(v for n, v in phases.items() if n.startswith("cart_"))
    out = {n: round(v, 4) for n, v in t.items()}
    out["ours_iteration_operator_ms"] = round(ours_iter, 4)
    out["speedup_forward"] = round(t["cufft_forward_ms"] / t["ours_forward_ms"], 2)
    out["speedup_adjoint"] = round(t["cufft_adjoint_ms"] / t["ours_adjoint_ms"], 2)
    out["speedup_iteration_operator"] = round(t["cufft_iteration_operator_ms"] / ours_iter, 2)
    out["note"] = ("ours forward writes the full masked k-space and adjoint reads it (as the reference API); "
                   "the iteration operator touches only sampled columns")
    return out


def run_ncu_case(args):
    """The workload's kernels for an ncu capture: operator set-up, autotuning and graph capture run first,
    then one solve of --ncu-iters iterations runs between cudaProfilerStart and cudaProfilerStop, so
    `ncu --profile-from-start off` sees exactly those launches (5 kernels per Cartesian iteration, 9 per
    radial iteration)."""
    import torch

    import primaldualtoolbox as pdt

    stream = torch.cuda.current_stream()
    if args.ncu_workload == "cnn":
        # the warm-start network: one training step (forward, backward, Adam) on a batch of 4 images of
        # 320 x 320 (the learned-warm-start configuration), --ncu-iters times between the profiler marks
        from primaldualtoolbox import warmstart

        rng = np.random.default_rng(0)

        def img(*shape):
            return torch.from_numpy((rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
                                    .astype(np.complex64)).cuda()

        net = warmstart.WarmStartNet(seed=0)
        u0, ut, vt = img(4, 320, 320), img(4, 320, 320), img(4, 2, 320, 320)
        for _ in range(3):
            net.train_step(u0, ut, vt, lr=1e-4, stream=stream)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        for _ in range(args.ncu_iters):
            net.train_step(u0, ut, vt, lr=1e-4, stream=stream)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"ncu_case": "warmstart_cnn_train_step_4x320x320", "steps": args.ncu_iters}), flush=True)
        return
    if args.ncu_workload == "batched":
        # the config-3 batch: --batch-cases mixed problems (the bench's batched leg), one batched solve of
        # --ncu-iters iterations per problem between the profiler marks
        import concurrent.futures
        import multiprocessing

        from primaldualtoolbox import warmstart

        specs = _batch_specs(args.batch_cases)
        with concurrent.futures.ProcessPoolExecutor(max(1, min(16, (os.cpu_count() or 2) - 1)),
                                                    mp_context=multiprocessing.get_context("spawn")) as pool:
            cases = list(pool.map(warmstart._case, specs, chunksize=1))
        opts = []
        for case in cases:
            op = pdt.mri.MriCartesianOperator()
            op.setCoilSens(case["sens"])
            op.setMask(case["mask"])
            opt = pdt.mri.TgvMriOptimizer_2c3c()
            prm = opt.getParameters()
            prm.max_iter, prm.reduction, prm.alpha1 = args.ncu_iters - 1, REDUCTION, case["alpha1"]
            prm.alpha0 = 2 * prm.alpha1
            opt.setOperator(op)
            opt.setNoisyData(case["rawdata"])
            opts.append(opt)
        del cases
        batch = pdt.batch.BatchSolver(opts)
        for _ in range(3):
            batch.solve(stream=stream)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        batch.solve(stream=stream)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"ncu_case": f"batch_{args.batch_cases}_cartesian_tgv2_mixed", "iterations": args.ncu_iters,
                          "shapes": [[s["C"], s["H"], s["W"]] for s in specs]}), flush=True)
        return
    if args.ncu_workload == "radial":
        op, f, a1 = _radial_problem(pdt, seed=0)
        opt = pdt.mri.TgvMriOptimizer_2c2c()
        prm = opt.getParameters()
        prm.max_iter, prm.reduction, prm.alpha1 = args.ncu_iters - 1, 2.0 ** -8, a1
        prm.alpha0 = 2 * a1
        opt.setOperator(op)
        opt.setNoisyData(f)
        for _ in range(3):
            opt.solve(stream=stream)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        opt.solve(stream=stream)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"ncu_case": "radial_tgv2_12c_256x256_64spokes_x512", "iterations": args.ncu_iters}),
              flush=True)
        return
    case = _problem(seed=0)
    dev = {k: torch.from_numpy(np.ascontiguousarray(case[k])).cuda() for k in ("rawdata", "sens", "mask")}
    op = pdt.mri.MriCartesianRemoveROOSOperator()
    op.setCoilSens(dev["sens"])
    op.setMask(dev["mask"])
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.max_iter, prm.reduction, prm.alpha1 = args.ncu_iters - 1, REDUCTION, case["alpha1"]
    prm.alpha0 = 2 * prm.alpha1
    opt.setOperator(op)
    opt.setNoisyData(dev["rawdata"], stream=stream)
    for _ in range(3):
        opt.solve(stream=stream)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    opt.solve(stream=stream)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"ncu_case": WORKLOAD, "iterations": args.ncu_iters, "tuning": op.tuning()}), flush=True)


def run_reference(args):
    """--impl reference: the reference's TGV-MRI iteration on the host cores. The reference's own CUDA
    build needs ImageUtilities, which it does not ship, so this is the CPU restatement of its iteration
    (FP32 mirror of tgvmrioptimizer.cu:120-200, all threads). Each step times a bounded sample of the
    1001-iteration solve: REF_SAMPLE_ITERS iterations from u0 = A^H f (the one-off A^H f outside the
    sample). Only numpy and the oracle are loaded here -- no part of this repository's GPU engine."""
    rank, world, _ = _rank_info()
    if rank != 0:
        return None
    from oracle import oracle

    case = _problem(seed=0)
    threads = os.cpu_count()
    oracle.set_threads(threads)
    u0 = oracle.op_apply("cartesian_roos", case["sens"], case["mask"], case["rawdata"], adjoint=True, prec=32)

    def step():
        oracle.op_solve("cartesian_roos", case["sens"], case["mask"], case["rawdata"], "tgv_mri",
                        alpha0=case["alpha0"], alpha1=case["alpha1"], reduction=REDUCTION,
                        max_iter=REF_SAMPLE_ITERS - 1, u0=u0, prec=32)

    for _ in range(min(args.warmup, 1)):  # the host path has nothing to warm beyond the first call
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    val = REF_SAMPLE_ITERS * args.steps / dt
    line = {"metric": METRIC, "value": round(val, 3), "unit": "iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic", "impl": "reference",
            "config": _config(case, world),
            "cpu_baseline": {"value": round(val, 3), "unit": "iters/s", "cores": threads, "kind": "port",
                             "sample": f"{REF_SAMPLE_ITERS} of the {ITERS} iterations per step, from u0 = A^H f "
                                       f"(computed once, outside the timed region), FP32 mirror of the "
                                       f"reference iteration"},
            "e2e": {"value": round(val, 3), "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--accuracy", type=int, default=1, help="measure iterations/time to rel-L2 1e-4 (1) or skip (0)")
    ap.add_argument("--stream-slices", type=int, default=12, help="streamed e2e leg: slices (0 skips)")
    ap.add_argument("--radial-slices", type=int, default=32, help="radial leg (config 5): slices (0 skips)")
    ap.add_argument("--denoising", type=int, default=1, help="TV-ROF / TGV denoising leg (config 1): 1 runs it")
    ap.add_argument("--cufft", type=int, default=1, help="time the Cartesian operator beside cuFFT (1) or skip (0)")
    ap.add_argument("--radial-iters", type=int, default=200, help="radial leg: iterations per slice")
    ap.add_argument("--batch-cases", type=int, default=64, help="batched leg: independent problems (0 skips)")
    ap.add_argument("--batch-iters", type=int, default=200, help="batched leg: iterations per problem and step")
    ap.add_argument("--ncu-workload", default="cartesian", choices=["cartesian", "radial", "cnn", "batched"],
                    help="profiling mode: the config-2 Cartesian problem, the config-5 radial slice, one "
                         "training step of the warm-start network or the config-3 batch (--batch-cases)")
    ap.add_argument("--ncu-iters", type=int, default=0,
                    help="profiling mode: one solve of this many iterations between cudaProfilerStart/Stop")
    args = ap.parse_args()
    if args.ncu_iters > 0:
        run_ncu_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
