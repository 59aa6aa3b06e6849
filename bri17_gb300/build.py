"""Builds the in-tree CUDA library ``bri17_gb300/libbri17_gb300.so``.

Each ``csrc/*.cu`` / ``csrc/*.cpp`` translation unit compiles in parallel
with nvcc for sm_103a only, then links into one shared library with the C ABI
of ``include/bri17_gb300.h``.  Objects go to ``bri17_gb300/_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbri17_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
              "-I", os.path.join(REPO, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(REPO, "include", "bri17_gb300.h"))
    return max(os.path.getmtime(h) for h in hs)


def _flags_tag(extra) -> str:
    """Object-name suffix for extra nvcc flags, so that objects built with
    other flags are never reused."""
    if not extra:
        return ""
    import hashlib
    return "." + hashlib.sha1("\0".join(extra).encode()).hexdigest()[:10]


def _compile(src: str, extra) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + _flags_tag(extra) + ".o")
    if (os.path.exists(obj) and os.path.getmtime(obj) > os.path.getmtime(src)
            and os.path.getmtime(obj) > _headers_mtime()):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    # The library records the objects it was linked from; another set (other
    # sources or flags) relinks it.
    stamp = os.path.join(BUILD, "libbri17_gb300.objs")
    linked = open(stamp).read() if os.path.exists(stamp) else None
    if (not os.path.exists(LIB) or linked != "\n".join(objs)
            or max(os.path.getmtime(o) for o in objs) > os.path.getmtime(LIB)):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
        with open(stamp, "w") as f:
            f.write("\n".join(objs))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
