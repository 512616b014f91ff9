"""Builds the CUDA extension ``sgldbench_gb300/libsgld_gb300.so`` in-tree.

The library holds every kernel and the C ABI of ``include/sgld_gpu.h``; it is
compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``).
Translation units compile in parallel; the whole build takes well under a
minute.  Also builds the MEX gateway (``sgldbench_gb300/mex``) against a
caller-supplied ``mex.h`` directory when one is given.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsgld_gb300.so")
SOURCES = ["kernels_stencil.cu", "kernels_mg.cu", "kernels_asm.cu", "kernels_vec.cu", "kernels_mixed.cu", "kernels_topopt.cu", "kernels_df.cu", "kernels_principal.cu", "kernels_pde.cu", "kernels_mma.cu", "kernels_net.cu", "kernels_net_tc.cu", "sgld_net.cu", "sgld_learned.cu", "noalloc.cu", "kernels_cases.cu", "sgld_cases.cu",
           "sgld_api.cu", "sgld_topopt_api.cu"]
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(INCLUDE, "sgld_gpu.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [NVCC, *ARCH, *FLAGS, "-c", path, "-o", obj]
    if os.environ.get("SGLD_PTXAS_VERBOSE"):
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if (not os.path.exists(LIB)) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_harness() -> str:
    """The standalone C++ driver (harness/sgld_harness.cpp) linked to the library."""
    lib = build()
    out = os.path.join(HERE, "harness", "sgld_harness")
    src = os.path.join(HERE, "harness", "sgld_harness.cpp")
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(src), os.path.getmtime(lib)):
        cmd = ["g++", "-O2", "-std=c++17", "-I", INCLUDE, src, "-o", out, "-L", HERE, "-lsgld_gb300",
               f"-Wl,-rpath,{HERE}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"harness build failed:\n{r.stderr}")
    return out


def build_mex_gateway(mex_include: str, out: str) -> str:
    """Compiles the MEX gateway (mex/sgld_gpu_mex.cpp) against the mex.h found
    in `mex_include`, with its entry point renamed to sgld_gpu_mex, into the
    shared object `out` linked to the library.  MATLAB users build it with
    MATLAB's own `mex` command instead."""
    lib = build()
    src = os.path.join(HERE, "mex", "sgld_gpu_mex.cpp")
    extra = [os.path.join(mex_include, f) for f in os.listdir(mex_include) if f.endswith(".cpp")]
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-DmexFunction=sgld_gpu_mex", "-I", mex_include,
           "-I", INCLUDE, src, *extra, "-o", out, "-L", HERE, "-lsgld_gb300", f"-Wl,-rpath,{HERE}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"MEX gateway build failed:\n{r.stderr}")
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    if "--harness" in sys.argv:
        print(build_harness())
