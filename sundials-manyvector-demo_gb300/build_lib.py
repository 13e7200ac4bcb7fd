"""Build libgbmv.so (the C-ABI library of include/gbmv.h) in-tree with nvcc for sm_103a.

Each .cu under csrc/ is compiled to an object in parallel, then linked with `nvcc -shared`.
Objects and the library land in sundials-manyvector-demo_gb300/_build/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libgbmv.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    # largest first: the slowest units start at once and the short ones fill in around them
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu")]
    return sorted(srcs, key=lambda p: (-os.path.getsize(p), p))


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(PKG, "..", "include", "gbmv.h"))
    return max(os.path.getmtime(h) for h in hdrs)


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _deps()):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"]
    if verbose_ptxas:
        cmd[1:1] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose_ptxas and r.stderr:
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if force:
        for f in os.listdir(OUT):
            if f.endswith(".o"):
                os.remove(os.path.join(OUT, f))
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1, len(srcs)))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
