"""In-tree build of the CUDA libraries (nvcc, sm_103a only).

``build()`` compiles every ``csrc/*.cu`` translation unit into one shared
library, ``_build/libnbg.so``, exporting the C ABI declared in
``include/nbg.h`` (and the other ``include/*.h`` headers).  Translation units
compile in parallel; nothing outside this directory is written.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(BUILD, "libnbg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no multiply-add contraction, so every float operation rounds
# once exactly as in the CPU oracle and the reference's scalar C++.
# -Xcompiler -ffp-contract=off: the same for host code (gcc contracts a*b+c into
# fma by default on aarch64).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
# translation units built with nvcc's default contraction: device code that
# must round as the reference's own kernels (built with defaults) do
DEFAULT_CONTRACTION = {"nbg_decay.cu"}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build neuronbridge_gb300")
    return cand


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE) if h.endswith(".h")]
    headers += [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    srcs = sources()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    cc = nvcc()

    def compile_one(pair):
        src, obj = pair
        if not force and not _stale(obj, [src] + headers):
            return None
        flags = NVCC_FLAGS
        if os.path.basename(src) in DEFAULT_CONTRACTION:
            flags = [f for f in NVCC_FLAGS if f != "-fmad=false"]
        cmd = [cc, *ARCH, *flags, *(extra or []), "-I", INCLUDE, "-c", src, "-o", obj + ".tmp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        os.replace(obj + ".tmp", obj)
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        logs = list(ex.map(compile_one, zip(srcs, objs)))
    if verbose:
        for lg in logs:
            if lg:
                print(lg, file=sys.stderr)
    if force or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
