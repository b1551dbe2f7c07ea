"""Builds libtay_gb300.so in-tree: CUDA kernels for sm_103a plus the host C layer.

    python -m tay_gb300._build [--verbose]

Each translation unit is compiled in parallel with nvcc (one -gencode, sm_103a) or gcc,
then linked with nvcc into tay_gb300/libtay_gb300.so.  Objects go to tay_gb300/_build/.
Host code is portable C/C++ (x86_64 here, aarch64 on Grace).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtay_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

GENCODE = "arch=compute_103a,code=sm_103a"
CU_SOURCES = [
    "gpu/sort.cu",
    "gpu/runtime.cu",
    "gpu/model_test_basic.cu",
    "gpu/model_box.cu",
    "gpu/model_boids.cu",
    "gpu/model_sph.cu",
    "gpu/noalloc.cu",
    "gpu/adjoint.cu",
]
C_SOURCES = [
    "host/tay_state.c",
]


def nvcc_path() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _newer(src_list, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_list)


def _deps(src):
    d = os.path.dirname(src)
    hdrs = [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cuh", ".h"))]
    hdrs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return [src] + hdrs


def build(verbose: bool = False, ptxas_verbose: bool = False, jobs: int = 0) -> str:
    nvcc = nvcc_path()
    os.makedirs(OBJ, exist_ok=True)
    cu_flags = ["-gencode", GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                "-I", INCLUDE, "--expt-relaxed-constexpr"]
    if ptxas_verbose:
        cu_flags += ["-Xptxas", "-v"]
    c_flags = ["-O2", "-std=gnu11", "-fPIC", "-Wall", "-I", INCLUDE]
    tasks = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(obj)
        if ptxas_verbose or _newer(_deps(src), obj):
            tasks.append([nvcc] + cu_flags + ["-c", src, "-o", obj])
    for s in C_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(obj)
        if _newer(_deps(src), obj):
            tasks.append(["gcc"] + c_flags + ["-c", src, "-o", obj])
    outputs = []
    if tasks:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(tasks), os.cpu_count() or 4)) as ex:
            outputs = list(ex.map(lambda c: _run(c, verbose), tasks))
    if tasks or not os.path.exists(LIB):
        _run([nvcc, "-shared", "-o", LIB] + objs + ["-lcudart", "-ldl"], verbose)
    if ptxas_verbose:
        return "\n".join(outputs)
    return LIB


def build_model(src: str, out: str, verbose: bool = False, defines=()) -> str:
    """Compiles a host's own device model (a .cu written against include/tay_gpu_model.cuh)
    into the shared library `out`, for tgpu_register_model_library.  Rebuilt only when the
    source or the engine's headers are newer.  `defines`: extra -D options."""
    gpu = os.path.join(CSRC, "gpu")
    deps = [src] + [os.path.join(gpu, f) for f in os.listdir(gpu) if f.endswith(".cuh")]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    if not _newer(deps, out):
        return out
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    _run([nvcc_path(), "-gencode", GENCODE, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
          "-Xcompiler", "-fPIC", "-shared", "--cudart", "shared", "-I", INCLUDE, "-I", gpu] +
         ["-D" + d for d in defines] + [src, "-o", out], verbose)
    return out


if __name__ == "__main__":
    out = build(verbose="--verbose" in sys.argv, ptxas_verbose="--ptxas" in sys.argv)
    print(out)
