"""Builds libgdtgb300.so in-tree: one nvcc per translation unit (in parallel), sm_103a only."""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libgdtgb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = _headers()
    objs = []
    todo = []
    for src in sources:
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            todo.append((src, obj))

    def compile_one(item):
        src, obj = item
        cmd = [NVCC] + FLAGS + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        return obj

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(compile_one, todo))
    if todo or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_examples(verbose)
    return LIB


def build_examples(verbose: bool = False):
    """C++ drivers over the C++ facade (cpp/gdt_gb300.hh), linked against the in-tree library."""
    cuda = os.path.dirname(os.path.dirname(NVCC))
    cpp = os.path.join(PKG, "cpp")
    out = []
    for src in sorted(glob.glob(os.path.join(cpp, "*.cc"))):
        exe = os.path.join(OUT, os.path.basename(src)[:-3])
        deps = [src, LIB] + glob.glob(os.path.join(cpp, "*.hh")) + _headers()
        if _stale(exe, deps):
            cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), "-I" + cpp,
                   "-I" + os.path.join(cuda, "include"), src, "-L" + OUT, "-lgdtgb300",
                   "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN", "-o", exe]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"example build failed:\n{r.stdout}\n{r.stderr}")
        out.append(exe)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
