"""Builds libsph_gb300.so in-tree: every translation unit compiled for
sm_103a by nvcc in parallel, then linked with the static CUDA runtime."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libsph_gb300.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["sph_kernels.cu", "sph_engine.cu", "sph_capi.cu", "sph_terrain.cpp", "sph_serve.cu", "sph_static.cu", "sph_recipe.cpp", "sph_mesh.cu",
           "sph_state.cu", "sph_gridcol.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off keeps host-side FP32 constants (kernel normalisations,
# terrain geometry) rounded exactly like the reference and the oracle on both
# x86-64 and aarch64 hosts.
HOST_FLAGS = "-fPIC,-ffp-contract=off,-O2,-fvisibility=hidden"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(HERE, "..", "include", "sph_erosion.h"))
    cmds = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            cmds.append([nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", HOST_FLAGS,
                         "-x", "cu", "-c", path, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, len(cmds))) as ex:
        list(ex.map(run, cmds))
    if cmds or not os.path.exists(OUT):
        tmp = OUT + ".tmp"
        subprocess.run([nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-cudart", "static", "-o", tmp, *objs,
                        "-lpthread"], check=True)
        os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
