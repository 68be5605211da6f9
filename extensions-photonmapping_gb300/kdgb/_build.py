"""In-tree build of libkdgb.so with nvcc for sm_103a.

The library is compiled from csrc/*.cu in parallel (one nvcc per translation
unit) and linked with `nvcc -shared`.  Arithmetic flags: --fmad=false keeps
every multiply and add separately rounded; -prec-div/-prec-sqrt give IEEE
division and square root; denormals are kept.  Objects go to csrc/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD_DIR = os.path.join(CSRC, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libkdgb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".hpp"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith((".h", ".hpp"))]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, obj: str, extra: list[str]) -> None:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")


def _machine_stamp_ok() -> bool:
    """Objects built on another host architecture are never reused."""
    stamp = os.path.join(BUILD_DIR, "HOST_ARCH")
    here = platform.machine()
    ok = os.path.exists(stamp) and open(stamp).read().strip() == here
    if not ok:
        with open(stamp, "w") as f:
            f.write(here + "\n")
    return ok


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compiles and links libkdgb.so if any source changed; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not _machine_stamp_ok():
        force = True
    extra = list(extra_flags or [])
    srcs = sources()
    hdrs = _headers()
    objs = [os.path.join(BUILD_DIR, os.path.basename(s)[:-3] + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, [s, *hdrs])]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            list(ex.map(lambda so: _compile(so[0], so[1], extra), todo))
    if force or todo or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    if verbose:
        print(f"libkdgb.so ready at {LIB_PATH}")
    return LIB_PATH


if __name__ == "__main__":
    import sys
    build(force="--force" in sys.argv, verbose=True)
