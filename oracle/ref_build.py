"""Build recipe for the REFERENCE tracer's host code (test infrastructure only).

The reference (meirbon/CudaTracer) is MSVC-only and does not compile unmodified
with g++: its binary BVH node puts an anonymous struct with glm members inside a
union (src/BVH/BVHNode.cuh:32-40), which g++ rejects ("member with constructor
not allowed in anonymous aggregate"). This recipe therefore

  1. copies the few source files the host BVH/camera path needs, plus the
     vendored header-only glm/assimp/GLFW headers, from the reference checkout
     into oracle/_ref/src and oracle/_ref/include (git-ignored build output);
  2. applies one mechanical patch that keeps the 32-byte layout:
       BVHNode.cuh  union{AABB bounds; struct{vec3 min; int leftFirst; vec3 max; int count;};}
                    -> AABB bounds;   (Intersect reads bounds.xMin.. / bounds.xMax..)
       BVHNode.cu   this->min[axis] -> bounds.bmin[axis]   (2 sites)
  3. compiles oracle/ref_harness.cpp with those sources into oracle/_ref/libctref.so,
     with -ffp-contract=off so no multiply-add is fused (matching the MSVC
     x86-64 build the reference targets).

Nothing produced here is committed. When the reference checkout is absent (the
GPU host), step 1-2 are skipped and an existing oracle/_ref/src (carried over
with the working tree) is compiled for the local architecture instead.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_OUT, "libctref.so")
# where the reference checkout is looked for: build(reference=...), then
# `--reference PATH` on the command line, then $CT_REFERENCE_DIR, then this
DEFAULT_REFERENCE = "/root/reference"

SRC_FILES = [
    "BVH/AABB.h", "BVH/BVHNode.cuh", "BVH/BVHNode.cu", "BVH/BVHTree.h", "BVH/BVHTree.cpp",
    "BVH/MBVHNode.cuh", "BVH/MBVHNode.cu", "BVH/MBVHTree.h", "BVH/MBVHTree.cpp",
    "Core/BSDF.h", "Core/Camera.h", "Core/Camera.cpp", "Core/Material.cuh", "Core/Microfacet.cuh",
    "Core/Random.cuh", "Core/Ray.cuh", "Core/SceneData.cuh", "Core/Tools.h", "Core/Triangle.cuh",
    "Core/TriangleList.h", "CUDA/CudaAssert.h", "Utils/ctpl.h", "Utils/Timer.h", "Utils/Surface.h",
]
INCLUDE_DIRS = ["glm", "assimp", "GLFW"]
COMPILED = ["BVH/BVHNode.cu", "BVH/BVHTree.cpp", "BVH/MBVHNode.cu", "BVH/MBVHTree.cpp", "Core/Camera.cpp"]

PATCHES = {
    "BVH/BVHNode.cuh": [
        (
            "\tunion {\n\t\tAABB bounds;\n\t\tstruct {\n\t\t\tglm::vec3 min;\n\t\t\tint leftFirst;\n"
            "\t\t\tglm::vec3 max;\n\t\t\tint count;\n\t\t};\n\t};\n",
            "\tAABB bounds;\n",
            1,
        ),
        (
            "const vec3 t1 = (this->min - org) * dirInverse;",
            "const vec3 t1 = (glm::vec3(bounds.xMin, bounds.yMin, bounds.zMin) - org) * dirInverse;",
            1,
        ),
        (
            "const vec3 t2 = (this->max - org) * dirInverse;",
            "const vec3 t2 = (glm::vec3(bounds.xMax, bounds.yMax, bounds.zMax) - org) * dirInverse;",
            1,
        ),
    ],
    "BVH/BVHNode.cu": [("this->min[axis]", "bounds.bmin[axis]", 2)],
}


# ---- the reference's own GPU frame (for the frame fixture, tests/golden/make_ref_frame.py)
#
# src/CUDA/Kernel.cu is built with nvcc from a patched copy of the whole src/
# tree under oracle/_ref/gpu/src. The patches are mechanical: they remove the
# OpenGL interop and the surface the viewer presents to (no graphics stack), let
# Camera-free device code see triangle::getBounds as host-only (its __m128 box
# type is host code), and replace the grid sizes n / 128 and n + n % 128 by
# ceil(n / 128): as written, the last n % 128 rays of a pass are dropped, and a
# bounce pass can read up to 127 rays past the end of its ray buffer; and the
# traversal stacks are enlarged from 32 to 64 entries (results are unchanged
# wherever 32 sufficed).
GPU_PATCHES = {
    "CUDA/Kernel.cuh": [
        ("#include <GL/glew.h>\n", "", 1),
        ("#include <cuda_gl_interop.h>\n", "", 1),
        ("\t\tint glDeviceId;\n\t\tunsigned int glDeviceCount;\n"
         "\t\tcudaGLGetDevices(&glDeviceCount, &glDeviceId, 1u, cudaGLDeviceListAll);\n",
         "\t\tint glDeviceId = 0;\n\t\tcudaGetDevice(&glDeviceId);\n", 1),
    ],
    "CUDA/Kernel.cu": [
        ("#include <surface_functions.h>\n", "", 1),
        ("#include <cuda_surface_types.h>\n", "", 1),
        ("surface<void, cudaSurfaceType2D> framebuffer;\n", "", 1),
        ("\tsurf2Dwrite(color, framebuffer, x * sizeof(vec4), y);\n", "", 1),
        ("\tsurf2Dwrite(color, framebuffer, x * sizeof(vec4), y, cudaBoundaryModeZero);\n", "", 1),
        ("\terr = cuda(BindSurfaceToArray(framebuffer, array));\n", "\terr = cudaSuccess;\n", 1),
        ("\tint groups = activePaths / 128;\n", "\tint groups = (activePaths + 127) / 128;\n", 1),
        ("const int shadowGroups = (connectCount + (connectCount % 128)) / 128;",
         "const int shadowGroups = (connectCount + 127) / 128;", 2),
        ("\t\tactivePaths = activePaths + (activePaths % 128);\n", "", 1),
        ("\t\tgroups = activePaths / 128;\n", "\t\tgroups = (activePaths + 127) / 128;\n", 1),
    ],
    "Core/Triangle.cuh": [
        ("\t__device__ __host__ inline static AABB getBounds(", "\t__host__ inline static AABB getBounds(", 1),
    ],
    "BVH/BVHNode.cuh": PATCHES["BVH/BVHNode.cuh"],
    "BVH/BVHNode.cu": PATCHES["BVH/BVHNode.cu"],
    # the traversal stacks hold 32 entries with no overflow check; a quad tree of
    # depth d needs up to 3d + 1 (43 for the 3.1 M-triangle terrain's depth 14)
    "BVH/MBVHNode.cuh": [
        ("\t\tMBVHTraversal todo[32];\n", "\t\tMBVHTraversal todo[64];\n", 3),
    ],
}
GPU_DIR = os.path.join(REF_OUT, "gpu")
GPU_LIB = os.path.join(REF_OUT, "libctref_gpu.so")


def stage_gpu_sources(reference: str) -> None:
    """Copy the reference's src/ tree to oracle/_ref/gpu/src and apply GPU_PATCHES."""
    dst = os.path.join(GPU_DIR, "src")
    if os.path.isdir(dst):
        shutil.rmtree(dst)
    shutil.copytree(os.path.join(reference, "src"), dst)
    for rel, patches in GPU_PATCHES.items():
        path = os.path.join(dst, rel)
        with open(path, "r", encoding="utf-8-sig", errors="replace") as f:
            text = _normalise(f.read())
        for old, new, count in patches:
            found = text.count(old)
            if found != count:
                raise RuntimeError(f"reference GPU patch for {rel}: expected {count} match(es), found {found}")
            text = text.replace(old, new)
        with open(path, "w", encoding="utf-8") as f:
            f.write(text)


def compile_gpu_lib(verbose: bool = False) -> str:
    """nvcc build of the patched Kernel.cu + Camera.cpp + oracle/ref_gpu_harness.cu into
    oracle/_ref/libctref_gpu.so (sm_103a). Needs oracle/_ref/gpu/src (staged from the
    reference checkout) and the staged headers in oracle/_ref/include."""
    src = os.path.join(GPU_DIR, "src")
    if not os.path.isdir(src):
        raise FileNotFoundError("oracle/_ref/gpu/src is missing: the reference checkout was never staged")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    shim = os.path.join(HERE, "ref_shim")
    flags = ["-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2", "-w", "-Xcompiler", "-fPIC",
             "-DGLM_FORCE_PURE", "-DGLEW_NO_GLU", "-DGLFW_INCLUDE_NONE",
             "-include", os.path.join(shim, "ct_ref_cuda_shim.h"), "-I", os.path.join(shim, "stub")]
    if not _is_x86():  # the box-type AABB's SSE intrinsics from the portable header
        flags += ["-I", os.path.join(shim, "portable")]
    flags += ["-I", src, "-I", os.path.join(REF_OUT, "include")]
    objs = []
    for p in (os.path.join(src, "CUDA", "Kernel.cu"), os.path.join(src, "Core", "Camera.cpp"),
              os.path.join(HERE, "ref_gpu_harness.cu")):
        obj = os.path.join(GPU_DIR, os.path.basename(p).replace(".", "_") + ".o")
        cmd = [nvcc] + flags + ["-x", "cu", "-c", p, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        objs.append(obj)
    cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", GPU_LIB] + objs
    subprocess.run(cmd, check=True)
    return GPU_LIB


def _normalise(text: str) -> str:
    return text.replace("\r\n", "\n")


def stage_sources(reference: str) -> None:
    src_out = os.path.join(REF_OUT, "src")
    inc_out = os.path.join(REF_OUT, "include")
    os.makedirs(src_out, exist_ok=True)
    for rel in SRC_FILES:
        with open(os.path.join(reference, "src", rel), "r", encoding="utf-8-sig", errors="replace") as f:
            text = _normalise(f.read())
        for old, new, count in PATCHES.get(rel, []):
            found = text.count(old)
            if found != count:
                raise RuntimeError(f"reference patch for {rel}: expected {count} match(es), found {found}")
            text = text.replace(old, new)
        dst = os.path.join(src_out, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        with open(dst, "w", encoding="utf-8") as f:
            f.write(text)
    for d in INCLUDE_DIRS:
        dst = os.path.join(inc_out, d)
        if os.path.isdir(dst):
            shutil.rmtree(dst)
        shutil.copytree(os.path.join(reference, "include", d), dst)


def _is_x86() -> bool:
    return platform.machine().lower() in ("x86_64", "amd64", "i686", "i386")


def compile_lib(verbose: bool = False) -> str:
    src_dir = os.path.join(REF_OUT, "src")
    if not os.path.isdir(src_dir):
        raise FileNotFoundError("oracle/_ref/src is missing: the reference checkout was never staged")
    harness = os.path.join(HERE, "ref_harness.cpp")
    inputs = [harness] + [os.path.join(src_dir, c) for c in COMPILED]
    newest = max(os.path.getmtime(p) for p in inputs + [os.path.abspath(__file__)])
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest and _lib_matches_arch(LIB):
        return LIB
    shim = os.path.join(HERE, "ref_shim")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    flags = [
        "-std=c++17", "-O2", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-w",
        "-DGLM_FORCE_PURE", "-DGLEW_NO_GLU", "-DGLFW_INCLUDE_NONE",
        "-include", os.path.join(shim, "ct_ref_shim.h"),
        "-I", os.path.join(shim, "stub"),
    ]
    if not _is_x86():
        flags += ["-I", os.path.join(shim, "portable")]
    flags += ["-I", src_dir, "-I", os.path.join(REF_OUT, "include"), "-I", cuda_inc]
    objs = []
    procs = []
    for p in inputs:
        obj = os.path.join(REF_OUT, os.path.basename(p).replace(".", "_") + ".o")
        cmd = ["g++"] + flags + ["-x", "c++", "-c", p, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), p))
        objs.append(obj)
    for proc, p in procs:
        out, _ = proc.communicate()
        if proc.returncode != 0:
            raise RuntimeError(f"compiling {p} failed:\n{out.decode(errors='replace')}")
    tmp = LIB + ".tmp"
    cmd = ["g++", "-shared", "-pthread", "-o", tmp] + objs
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def _lib_matches_arch(path: str) -> bool:
    try:
        with open(path, "rb") as f:
            head = f.read(20)
        machine = int.from_bytes(head[18:20], "little")
        return machine == (62 if _is_x86() else 183)  # EM_X86_64 / EM_AARCH64
    except OSError:
        return False


def build(reference: str | None = None, verbose: bool = False) -> str | None:
    """Stage (when the reference checkout exists) and compile; returns the .so path or None."""
    reference = reference or os.environ.get("CT_REFERENCE_DIR", DEFAULT_REFERENCE)
    if os.path.isdir(os.path.join(reference, "src", "BVH")):
        stage_sources(reference)
        stage_gpu_sources(reference)
    if not os.path.isdir(os.path.join(REF_OUT, "src")):
        return None
    return compile_lib(verbose=verbose)


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="stage and compile the reference's host BVH/camera code")
    ap.add_argument("--reference", default=None, help="reference checkout (default: $CT_REFERENCE_DIR or "
                                                      f"{DEFAULT_REFERENCE})")
    ap.add_argument("-v", action="store_true", help="print the compiler commands")
    a = ap.parse_args()
    print(build(reference=a.reference, verbose=a.v))
