"""Writes the golden vectors of the reference's own code: tests/golden/ref_small.npz and ref_config2.npz.

The outputs come from oracle/_ref/libpdtref.so -- the reference's optimizer loops, TGV kernels and
Cartesian operators (src/optimizer/*, src/operator/mricartesianoperator.cu) compiled for the CPU by
oracle/ref_build.py -- so this script needs the reference checkout:

    python tests/golden/make_ref_golden.py <path of the reference checkout>

ref_small.npz holds the inputs and outputs of small cases of every optimizer and of the two Cartesian
operators, plus the denoising benchmark (TV-ROF on the seeded 512 x 512 phantom, 501 iterations).
ref_config2.npz holds the result of the benchmark reconstruction itself (15 coils x 640 x 368 with
readout-oversampling removal, 1001 iterations, reduction 2e-8; about 15 minutes on 8 cores) and a
SHA-256 of its seeded inputs, which are regenerated by primaldualtoolbox/synthetic.py where they are used.
"""
import hashlib
import importlib.util
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT]


def _synthetic():
    spec = importlib.util.spec_from_file_location(
        "pdt_synthetic", os.path.join(ROOT, "primal-dual-toolbox_gb300", "primaldualtoolbox", "synthetic.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def small(ref, syn):
    out = {}
    f32 = np.float32
    # Cartesian operators, ROOS and plain
    for roos, (C, H, W) in ((True, (4, 64, 48)), (False, (3, 32, 24))):
        key = "roos" if roos else "cart"
        rng = np.random.default_rng(7 + roos)
        sens = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
        mask = (rng.random((H, W)) < 0.6).astype(np.float32)
        mask[:, rng.random(W) < 0.3] = 0
        Hi = H // 2 if roos else H
        u = (rng.standard_normal((Hi, W)) + 1j * rng.standard_normal((Hi, W))).astype(np.complex64)
        k = (rng.standard_normal((C, H, W)) + 1j * rng.standard_normal((C, H, W))).astype(np.complex64)
        out.update({f"op_{key}_sens": sens, f"op_{key}_mask": mask, f"op_{key}_u": u, f"op_{key}_k": k,
                    f"op_{key}_fwd": ref.cart_apply(roos, sens, mask, u),
                    f"op_{key}_adj": ref.cart_apply(roos, sens, mask, k, adjoint=True)})
    # TgvMriOptimizer: ROOS 4c 64 x 48 with the sample's schedule for 1001 iterations; plain 3c 32 x 48
    for key, C, H, W, roos, red, it in (("tgvmri_roos", 4, 64, 48, True, 2e-8, 1000),
                                        ("tgvmri_cart", 3, 32, 48, False, 0.1, 100)):
        c = syn.cartesian_case(C=C, H=H, W=W, roos=roos, seed=1)
        a1 = f32(c["alpha1"])
        a0 = f32(2 * a1)
        out.update({f"{key}_sens": c["sens"], f"{key}_mask": c["mask"], f"{key}_f": c["rawdata"],
                    f"{key}_params": np.array([a0, a1, f32(red), it], np.float64),
                    f"{key}_u": ref.tgv_mri(roos, c["sens"], c["mask"], c["rawdata"], a0, a1, f32(red), it)})
    # TgvOptimizerWithOp / TvOptimizerWithOp, plain Cartesian 3c 32 x 24, Lambda 2, 301 iterations
    c = syn.cartesian_case(C=3, H=32, W=24, roos=False, seed=3)
    out.update({"withop_sens": c["sens"], "withop_mask": c["mask"], "withop_f": c["rawdata"],
                "withop_alpha": np.array([f32(c["alpha0"]), f32(c["alpha1"])], np.float64)})
    out["tgvop_u"] = ref.with_op("tgv_op", False, c["sens"], c["mask"], c["rawdata"], 2.0, 300, f32(c["alpha0"]),
                                 f32(c["alpha1"]))
    out["tvop_u"] = ref.with_op("tv_op", False, c["sens"], c["mask"], c["rawdata"], 2.0, 300)
    # denoising: TV-ROF benchmark (512 x 512 float32, Lambda 10, 500 -> 501 iterations), TGV real / complex
    noisy, _ = syn.tv_phantom(512, 512, seed=0)
    noisy = noisy.astype(np.float32)
    out.update({"rof_f": noisy, "rof_u": ref.denoise("tv", noisy, 10.0, 500)})
    g = syn.tv_phantom(64, 80, seed=2)[0].astype(np.float32)
    gc = (g * np.exp(1j * np.linspace(0, 2, 80))[None, :]).astype(np.complex64)
    out.update({"tgv_f": g, "tgv_u": ref.denoise("tgv", g, 10.0, 200, alpha0=0.2, alpha1=0.1),
                "tgvc_f": gc, "tgvc_u": ref.denoise("tgv", gc, 10.0, 200, alpha0=0.2, alpha1=0.1),
                "tvc_u": ref.denoise("tv", gc, 10.0, 200)})
    return out


def config2(ref, syn):
    c = syn.cartesian_case(C=15, H=640, W=368, roos=True, seed=0)
    a1 = np.float32(c["alpha1"])
    t0 = time.perf_counter()
    u = ref.tgv_mri(True, c["sens"], c["mask"], c["rawdata"], np.float32(2 * a1), a1, np.float32(2e-8), 1000)
    return {"u": u, "inputs_sha256": np.array(digest(c["rawdata"], c["sens"], c["mask"])),
            "params": np.array([2 * a1, a1, np.float32(2e-8), 1000], np.float64),
            "seconds": time.perf_counter() - t0, "threads": os.cpu_count()}


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_ref_golden.py <path of the reference checkout> [small|config2]")
    os.environ["PDT_REFERENCE_DIR"] = sys.argv[1]
    from oracle import ref

    if not ref.available():
        sys.exit("the reference checkout could not be built")
    syn = _synthetic()
    which = sys.argv[2:] or ["small", "config2"]
    if "small" in which:
        np.savez_compressed(os.path.join(HERE, "ref_small.npz"), **small(ref, syn))
        print("ref_small.npz written")
    if "config2" in which:
        np.savez_compressed(os.path.join(HERE, "ref_config2.npz"), **config2(ref, syn))
        print("ref_config2.npz written")


if __name__ == "__main__":
    main()
