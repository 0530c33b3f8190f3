"""Build libgray_gb300.so in-tree with nvcc (sm_103a only, no cmake).

    python -m gray_gb300.build [--verbose-ptxas]

Each .cu file in gray_gb300/csrc/ is compiled in parallel to an object file and the objects are
linked into gray_gb300/_build/libgray_gb300.so.  `-fmad=false` keeps every float expression
evaluated as written (the kernels use explicit fmaf where an FMA is wanted), which is what makes
the results reproducible bit-for-bit by the CPU oracle.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgray_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fno-strict-aliasing"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_newer(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "gray_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose_ptxas: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    srcs = sources()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []

    def compile_one(src_obj):
        src, obj = src_obj
        if not force and not _deps_newer(obj, src):
            return ""
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        logs = list(ex.map(compile_one, zip(srcs, objs)))
    if verbose_ptxas:
        for src, log in zip(srcs, logs):
            if log:
                print(f"== {os.path.basename(src)}\n{log}")
    relink = force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)
    if relink:
        tmp = LIB + ".tmp"
        cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


TORCH_SRC = os.path.join(HERE, "torch_binding", "gray_torch.cpp")
TORCH_LIB = os.path.join(BUILD, "libgray.so")


def build_torch_binding(force: bool = False) -> str:
    """Build libgray.so: torch.classes.gray.* (the reference's TorchScript classes) over the C ABI,
    compiled with g++ against the installed torch and linked to libgray_gb300.so (found next to it)."""
    import torch
    from torch.utils import cpp_extension as ce

    lib = build(force=force)
    deps = [TORCH_SRC, lib, os.path.join(HERE, "..", "include", "gray_gb300.h")]
    if not force and os.path.exists(TORCH_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(TORCH_LIB)
                                                        for d in deps):
        return TORCH_LIB
    cuda_home = os.path.dirname(os.path.dirname(nvcc()))
    torch_lib = os.path.join(os.path.dirname(torch.__file__), "lib")
    incs = [f"-I{p}" for p in ce.include_paths()] + [f"-I{os.path.join(cuda_home, 'include')}"]
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    tmp = TORCH_LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-D_GLIBCXX_USE_CXX11_ABI={abi}", *incs, TORCH_SRC,
           "-o", tmp, f"-L{torch_lib}", "-lc10", "-lc10_cuda", "-ltorch_cpu", "-ltorch",
           f"-L{BUILD}", "-lgray_gb300", f"-L{os.path.join(cuda_home, 'lib64')}", "-lcudart",
           "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath,{torch_lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {TORCH_SRC}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, TORCH_LIB)
    return TORCH_LIB


if __name__ == "__main__":
    print(build(verbose_ptxas="--verbose-ptxas" in sys.argv, force="--force" in sys.argv))
    if "--torch-binding" in sys.argv:
        print(build_torch_binding(force="--force" in sys.argv))
