"""Build recipe for libdpca.so and the dpca command line (nvcc, sm_103a only).

Every translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a``; outputs land in
``distpca_gb300/_build/`` (git-ignored) and are rebuilt only when a source or
header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from typing import List

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdpca.so")
CLI = os.path.join(OUT, "dpca")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["k_stats.cu", "k_fp64.cu", "k_dense.cu", "k_mixed.cu", "k_gprod.cu", "k_fullsvd.cu", "k_windows.cu", "handle.cu"]
CPP_SOURCES = ["host.cpp", "serve.cpp", "eig_host.cpp", "rows.cpp"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _headers() -> List[str]:
    hs = [os.path.join(INCLUDE, "dpca.h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stale(target: str, deps: List[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, obj: str, verbose: bool) -> None:
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", "--expt-relaxed-constexpr", *common, "-c", src, "-o", obj]
        if os.environ.get("DPCA_PTXAS_V"):
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = [nvcc(), "-x", "c++", *common, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    tmp = obj + f".tmp{os.getpid()}"
    cmd[cmd.index(obj)] = tmp
    subprocess.check_call(cmd)
    os.replace(tmp, obj)


def build(verbose: bool = False, jobs: int = 0) -> str:
    """Compile libdpca.so and the dpca CLI; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    heads = _headers()
    objs = []
    work = []
    for s in CU_SOURCES + CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + heads):
            work.append((src, obj))
    if work:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(work), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_compile, s, o, verbose) for s, o in work]:
                f.result()
    if _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        # cuSOLVER (dense eigensolve of the -fullSVD check) is a shared library of the toolkit
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "lib64")
        subprocess.check_call([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lcusolver",
                               "-Xlinker", f"-rpath={cuda_lib}", "-lrt", "-ldl", "-lpthread"])
        os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "cli.cpp")
    if _stale(CLI, [cli_src, LIB] + heads):
        tmp = CLI + f".tmp{os.getpid()}"
        subprocess.check_call([nvcc(), "-x", "c++", "-O2", "-std=c++17", "-I", INCLUDE, cli_src, "-o", tmp, "-L", OUT,
                               "-ldpca", "-Xlinker", "-rpath=$ORIGIN"])
        os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
