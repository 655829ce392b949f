"""Builds oracle/_ref/libpdtref.so: the reference's own optimizer loops, TGV kernels and Cartesian operators,
compiled for the CPU.

TEST INFRASTRUCTURE ONLY. The library pins the oracle restatement (oracle/pdt_oracle.cpp) and writes the
golden vectors in tests/golden/; nothing of the product loads it.

Recipe (no CMake, nothing of the reference's own build): the reference's source files on this path --
src/optimizer/{tgv_kernels.cuh, optimizer_helper.h, t*optimizer*.{h,cu}}, src/operator/{operatorbase.h,
mricartesianoperator.{h,cu}}, src/{definitions.h, iurandom.h, primaldualtoolbox_api.h} -- are read from
the reference checkout and written to oracle/_ref/gen/ with one mechanical change: every CUDA launch
`kernel<<<grid, block>>>(args);` becomes `pdtref::launch(grid, block, [&]() { kernel(args); });`, which
runs the kernel body once per (block, thread) on the host (oracle/ref_shim/iu/pdt_iu_shim.h; the kernels
on this path use no shared memory and no block barriers). Nothing else of the sources is changed. They
compile with g++ against oracle/ref_shim/, the host stand-in for ImageUtilities (an empty submodule in
the reference checkout), and link with oracle/ref_driver.cpp, a C entry point per optimizer and operator.
The generated sources stay under oracle/_ref/ (git-ignored); the reference's sources are not copied into
the repository.

    python oracle/ref_build.py [reference checkout]      (default: /root/reference)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
GEN = os.path.join(OUT, "gen")
LIB = os.path.join(OUT, "libpdtref.so")
DEFAULT_REFERENCE = "/root/reference"

SOURCES = [
    "src/definitions.h", "src/iurandom.h", "src/primaldualtoolbox_api.h",
    "src/operator/operatorbase.h", "src/operator/mricartesianoperator.h", "src/operator/mricartesianoperator.cu",
    "src/optimizer/optimizer_helper.h", "src/optimizer/tgv_kernels.cuh",
    "src/optimizer/tvoptimizer.h", "src/optimizer/tvoptimizer.cu",
    "src/optimizer/tgvoptimizer.h", "src/optimizer/tgvoptimizer.cu",
    "src/optimizer/tvoptimizerwithop.h", "src/optimizer/tvoptimizerwithop.cu",
    "src/optimizer/tgvoptimizerwithop.h", "src/optimizer/tgvoptimizerwithop.cu",
    "src/optimizer/tgvmrioptimizer.h", "src/optimizer/tgvmrioptimizer.cu",
]
UNITS = [s for s in SOURCES if s.endswith(".cu")]


def _split_top(s: str) -> list[str]:
    """Split on commas outside parentheses / brackets / angle brackets."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([<{":
            depth += 1
        elif ch in ")]>}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    return [x.strip() for x in out]


def rewrite_launches(text: str) -> tuple[str, int]:
    """`K<T> <<<g, b>>>(args);` -> `pdtref::launch(g, b, [&]() { K<T>(args); });` for every launch."""
    n = 0
    while True:
        i = text.find("<<<")
        if i < 0:
            return text, n
        j = text.index(">>>", i)
        # the kernel expression: back to the start of the statement
        k = max(text.rfind(";", 0, i), text.rfind("{", 0, i), text.rfind("}", 0, i)) + 1
        seg = text[k:i]
        kernel = seg.strip().split("\n")[-1].strip()  # comment lines before the launch stay where they are
        k += seg.rindex(kernel)
        params = _split_top(text[i + 3:j])
        a = text.index("(", j)
        depth, e = 0, a
        while True:
            if text[e] == "(":
                depth += 1
            elif text[e] == ")":
                depth -= 1
                if depth == 0:
                    break
            e += 1
        semi = text.index(";", e)
        args = text[a + 1:e]
        repl = f"pdtref::launch({params[0]}, {params[1]}, [&]() {{ {kernel}({args}); }});"
        text = text[:k] + repl + text[semi + 1:]
        n += 1


def generate(ref: str) -> list[str]:
    units = []
    for rel in SOURCES:
        src = os.path.join(ref, rel)
        text = open(src, encoding="utf-8").read()
        text, n = rewrite_launches(text)
        dst_rel = rel[len("src/"):]
        if dst_rel.endswith(".cu"):
            dst_rel = dst_rel[:-3] + ".cpp"
            units.append(os.path.join(GEN, dst_rel))
        dst = os.path.join(GEN, dst_rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        with open(dst, "w", encoding="utf-8") as fh:
            fh.write(f"// generated by oracle/ref_build.py from the reference's {rel} ({n} launches rewritten)\n")
            fh.write(text)
    return units


def _flags():
    return ["-O2", "-std=c++17", "-fopenmp", "-fPIC", "-ffp-contract=off", "-w", "-I", os.path.join(HERE, "ref_shim"),
            "-I", GEN, "-I", os.path.join(GEN, "operator"), "-I", os.path.join(GEN, "optimizer")]


def build(ref: str | None = None, force: bool = False) -> str | None:
    """Builds the library if the reference checkout exists; returns its path, or None without a checkout."""
    ref = ref or os.environ.get("PDT_REFERENCE_DIR") or DEFAULT_REFERENCE
    if not os.path.isdir(os.path.join(ref, "src", "optimizer")):
        return None
    deps = [os.path.join(ref, s) for s in SOURCES] + [
        os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "ref_shim", "iu", "pdt_iu_shim.h"), __file__]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    os.makedirs(GEN, exist_ok=True)
    units = generate(ref) + [os.path.join(HERE, "ref_driver.cpp")]

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        r = subprocess.run(["g++"] + _flags() + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"g++ failed for {src}:\n{r.stderr[-4000:]}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB + ".tmp"
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    path = build(sys.argv[1] if len(sys.argv) > 1 else None, force=True)
    print(path or "reference checkout not found: nothing built")
