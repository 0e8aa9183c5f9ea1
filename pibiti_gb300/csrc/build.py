"""Build recipe for libpibiti_sph.so (the C-ABI library) with nvcc.

Every translation unit is compiled for sm_103a only, in parallel, then
linked into ``pibiti_gb300/_lib/libpibiti_sph.so`` (in-tree, git-ignored).
The CUDA sources are built with ``--fmad=false``: the kernels spell out every
fused multiply-add they want, so the compiler must not add others.

Run as ``python -m pibiti_gb300.csrc.build`` or call ``build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libpibiti_sph.so")

CUDA_SOURCES = ["sph_stage.cu", "sph_scan.cu", "sph_system.cu", "sph_noalloc.cu", "sph_mlp.cu",
                "sph_render.cu"]
HOST_SOURCES = ["scene.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _flags(verbose_ptxas: bool, defines=()):
    f = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
         "-I", os.path.join(ROOT, "include"), "-I", HERE]
    f += [f"-D{d}" for d in defines]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src: str, obj: str, cuda: bool, verbose_ptxas: bool, defines=()) -> str:
    cmd = [nvcc(), "-c", os.path.join(HERE, src), "-o", obj] + _flags(verbose_ptxas, defines)
    if cuda:
        cmd += ARCH
    else:
        cmd += ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(HERE, f) for f in os.listdir(HERE)
            if f.endswith((".cu", ".cuh", ".cpp", ".h"))]
    deps += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False, defines=(), out: str = None) -> str:
    """Build the library; `defines` (NAME=VALUE strings) and `out` (another
    library path) build a variant, e.g. another launch shape for the walks."""
    lib = out or LIB
    if not force and out is None and not defines and not _stale():
        return LIB
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    objdir = lib + ".obj"
    os.makedirs(objdir, exist_ok=True)
    jobs = [(s, os.path.join(objdir, s + ".o"), True) for s in CUDA_SOURCES]
    jobs += [(s, os.path.join(objdir, s + ".o"), False) for s in HOST_SOURCES]
    logs = {}
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        futs = {ex.submit(_compile, s, o, c, verbose_ptxas, defines): s for s, o, c in jobs}
        for f in cf.as_completed(futs):
            logs[futs[f]] = f.result()
    tmp = lib + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + [o for _, o, _ in jobs] + ARCH + ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose_ptxas:
        for s, log in sorted(logs.items()):
            sys.stderr.write(f"== {s}\n{log}")
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
