"""Build recipe of the CUDA library: every ``csrc/*.cu`` compiled for sm_103a in parallel,
linked into ``scihpc_gb300/_lib/libscihpc_gb300.so`` (in-tree, git-ignored); then the C++
API layer (``cpp/scihpc_cpp.cpp``, the reference's class names over the C ABI) into
``scihpc_gb300/_lib/libscihpc_cpp.so``.

    python -m scihpc_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libscihpc_gb300.so")
CPP_SRC = os.path.join(HERE, "cpp", "scihpc_cpp.cpp")
CPP_INC = os.path.join(HERE, "cpp")
CPP_LIB = os.path.join(OUT, "libscihpc_cpp.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"),
         "--expt-relaxed-constexpr"]


# Per-file flags: the boundary fills must round exactly like the reference's separate
# multiply and add, so contraction into fused multiply-adds is off there.
FILE_FLAGS = {"bc.cu": ["-fmad=false"], "transport.cu": ["-fmad=false"], "secorder.cu": ["-fmad=false"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def cxx_flags() -> list[str]:
    """Flags for host C++ that uses the C++ API layer (headers, library, CUDA runtime)."""
    cuda = cuda_home()
    return ["-std=c++17", "-I" + CPP_INC, "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"),
            "-L" + OUT, "-lscihpc_cpp", "-lscihpc_gb300", "-L" + os.path.join(cuda, "lib64"), "-lcudart",
            "-Wl,-rpath," + OUT]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(SRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(SRC, "*.cuh"))) + [os.path.join(ROOT, "include", "scihpc_gpu.h"),
                                                                os.path.abspath(__file__)]
    cc = nvcc()
    jobs = []
    objs = []
    for s in sources:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc, *ARCH, *FLAGS, *FILE_FLAGS.get(os.path.basename(s), []), "-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build step failed: {' '.join(cmd[:3])} ...:\n{r.stdout}\n{r.stderr}")
        return r

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    cpp_deps = [CPP_SRC, LIB, os.path.abspath(__file__)] + sorted(glob.glob(os.path.join(CPP_INC, "scihpc", "*.h")))
    if force or _stale(CPP_LIB, cpp_deps):
        cuda = cuda_home()
        run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall", "-I" + CPP_INC,
             "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"), CPP_SRC, "-o", CPP_LIB,
             "-L" + OUT, "-lscihpc_gb300", "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + OUT])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
