"""Writes tests/golden/config2_fp64.npz: the FP64 CPU oracle's solution of the benchmark problem.

The problem is the 15-coil 640 x 368 Cartesian TGV-MRI reconstruction with readout-oversampling removal
on the seeded synthetic case (primaldualtoolbox.synthetic.cartesian_case, seed 0), solved as the
reference's sample does: max_iter = 1000 (1001 iterations), alpha continuation reduction 2e-8,
alpha0 = 2 alpha1, from u0 = A^H f. The oracle runs in double precision (about 7 minutes on 8 cores).
bench.py reports the rel-L2 distance of its GPU result to this solution. The file also holds a SHA-256
of the generated inputs, so a machine whose numpy generates different inputs is detected.

    python tests/golden/make_config2_fp64.py
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "primal-dual-toolbox_gb300"), ROOT]

C, H, W = 15, 640, 368
MAX_ITER, REDUCTION = 1000, 2e-8


def inputs_digest(case):
    h = hashlib.sha256()
    for k in ("rawdata", "sens", "mask"):
        h.update(np.ascontiguousarray(case[k]).tobytes())
    return h.hexdigest()


def main():
    import importlib.util

    from oracle import oracle

    # the phantom generator alone (numpy only), without loading the GPU library
    spec = importlib.util.spec_from_file_location(
        "pdt_synthetic", os.path.join(ROOT, "primal-dual-toolbox_gb300", "primaldualtoolbox", "synthetic.py"))
    synthetic = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(synthetic)

    case = synthetic.cartesian_case(C=C, H=H, W=W, roos=True, seed=0)
    oracle.set_threads(os.cpu_count())
    t0 = time.perf_counter()
    u = oracle.op_solve("cartesian_roos", case["sens"], case["mask"], case["rawdata"], "tgv_mri",
                        alpha0=float(np.float32(2 * np.float32(case["alpha1"]))),
                        alpha1=float(np.float32(case["alpha1"])), reduction=float(np.float32(REDUCTION)),
                        max_iter=MAX_ITER, prec=64)
    dt = time.perf_counter() - t0
    np.savez_compressed(os.path.join(HERE, "config2_fp64.npz"), u=u.astype(np.complex64),
                        inputs_sha256=np.array(inputs_digest(case)), max_iter=MAX_ITER, reduction=REDUCTION,
                        alpha1=np.float32(case["alpha1"]), seconds=dt, threads=os.cpu_count())
    print(f"config2_fp64.npz written ({dt:.0f} s on {os.cpu_count()} threads)")


if __name__ == "__main__":
    main()
