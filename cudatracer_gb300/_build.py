"""In-tree build of libcudatracer.so for sm_103a (nvcc, one -gencode, parallel TUs).

    python -m cudatracer_gb300._build        # or cudatracer_gb300._build.build()

Produces cudatracer_gb300/libcudatracer.so next to this file. Each translation
unit is compiled separately and in parallel; k_shade_exact.cu is compiled with
-fmad=false (its results are reproduced bit for bit by the CPU oracle), and
all host code with -ffp-contract=off (GCC fuses multiply-adds by default on
aarch64).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcudatracer.so")

SOURCES = {
    "api.cpp": [],
    "bvh_build.cpp": [],
    "bvh_fast.cpp": [],
    "mesh_io.cpp": [],
    "server.cpp": [],
    "k_trace.cu": [],
    "bvh_gpu.cu": [],
    "bvh_gpu_fast.cu": ["-fmad=false"],
    "k_trace_wide.cu": [],
    "k_shade_exact.cu": ["-fmad=false"],
    "k_shade_fast.cu": [],
    "noalloc.cu": [],
}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.exists(os.path.join(home, "bin", "nvcc")):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _inputs() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "cudatracer.h"))
    files.append(os.path.abspath(__file__))
    return files


def _up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    try:
        with open(LIB, "rb") as f:
            machine = int.from_bytes(f.read(20)[18:20], "little")
    except OSError:
        return False
    import platform

    want = 62 if platform.machine().lower() in ("x86_64", "amd64") else 183
    if machine != want:
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _inputs())


def build(verbose: bool = False, force: bool = False) -> str:
    if not force and _up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-Xcompiler", "-fno-fast-math", "-I", CSRC, "-I", os.path.join(ROOT, "include")] + ARCH

    def compile_one(item):
        src, extra = item
        obj = os.path.join(BUILD, src.replace(".", "_") + ".o")
        cmd = [nvcc] + common + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{p.stdout.decode(errors='replace')}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES.items()))
    tmp = LIB + ".tmp"
    libdir = os.path.join(home, "lib64")
    cmd = [nvcc, "-shared"] + ARCH + ["-cudart", "shared", "-o", tmp] + objs + [
        "-Xlinker", "-rpath", "-Xlinker", libdir, "-Xcompiler", "-pthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stdout.decode(errors='replace')}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
