"""Builds libradiantium_gb300.so in-tree for sm_103a.

Translation units compiled in parallel and linked with nvcc:
  rt_kernels.cu, rt_wavefront.cu, rt_adjoint.cu, rt_particles.cu  device code: --fmad=false keeps every
                 multiply and add separately rounded (the reference's
                 arithmetic), IEEE division and square root are nvcc's
                 defaults;
  rt_bvh_gpu.cu  the reference's SAH tree built on the GPU (--fmad=false:
                 bucket costs round like the host builder's);
  rt_noalloc.cu  the fixed scratch array of the allocation-free render;
  rt_host.cpp, rt_bvh.cpp  host runtime and BVH builder, -ffp-contract=off
                 for the same reason.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libradiantium_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def build(verbose: bool = False, extra_nvcc=(), extra_cxx=(), out_dir: str = OUT_DIR) -> str:
    """Compiles every translation unit in parallel and links the library into
    `out_dir`; returns the library's path.  A variant build (for example the
    debug-bounds one, extra_nvcc=["-DRT_DEBUG_BOUNDS"]) goes to its own out_dir."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(out_dir, exist_ok=True)
    lib = os.path.join(out_dir, os.path.basename(LIB))
    objs = {
        "rt_kernels.o": [nvcc, ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-warn-spills", *extra_nvcc, "-c", os.path.join(CSRC, "rt_kernels.cu")],
        "rt_wavefront.o": [nvcc, ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                            "-Xptxas", "-warn-spills", *extra_nvcc, "-c", os.path.join(CSRC, "rt_wavefront.cu")],
        "rt_adjoint.o": [nvcc, ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-warn-spills", *extra_nvcc, "-c", os.path.join(CSRC, "rt_adjoint.cu")],
        "rt_particles.o": [nvcc, ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                           "-Xptxas", "-warn-spills", *extra_nvcc, "-c", os.path.join(CSRC, "rt_particles.cu")],
        "rt_bvh_gpu.o": [nvcc, ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                         *extra_nvcc, "-c", os.path.join(CSRC, "rt_bvh_gpu.cu")],
        "rt_noalloc.o": [nvcc, ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *extra_nvcc,
                         "-c", os.path.join(CSRC, "rt_noalloc.cu")],
        "rt_host.o": ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", *extra_cxx,
                      f"-I{cuda}/include", "-c", os.path.join(CSRC, "rt_host.cpp")],
        "rt_bvh.o": ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                     "-c", os.path.join(CSRC, "rt_bvh.cpp")],
    }
    procs = []
    for obj, cmd in objs.items():
        full = cmd + ["-o", os.path.join(out_dir, obj)]
        if verbose:
            print(" ".join(full))
        procs.append((obj, subprocess.Popen(full, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for obj, p in procs:
        out, _ = p.communicate()
        if out and (verbose or p.returncode):
            sys.stdout.write(out)
        if p.returncode:
            failed.append(obj)
    if failed:
        raise RuntimeError(f"radiantium_gb300 build failed: {failed}")
    link = [nvcc, ARCH, "-shared", "-o", lib] + [os.path.join(out_dir, o) for o in objs] + ["-lpthread"]
    subprocess.run(link, check=True)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
