"""ctypes bindings to the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the checker for the GPU path: ``liboracle.so`` is the C
restatement in ``dpca_oracle.c`` (built here and on any machine that runs the
tests), and ``_ref/`` holds the unmodified reference built by
``build_ref.sh`` where the reference checkout exists.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_EXE = os.path.join(REF_DIR, "DistPCA.exe")
REF_HARNESS = os.path.join(REF_DIR, "ref_harness")


def build(force: bool = False) -> str:
    """Compile liboracle.so against scipy's OpenBLAS (seconds)."""
    src = os.path.join(HERE, "dpca_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    sys.path.insert(0, HERE)
    from find_openblas import find

    blas, ilp64 = find()
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I" + HERE] + (["-DDPCA_ORACLE_ILP64"] if ilp64 else [])
    cmd += [src, "-o", tmp, blas, "-Wl,-rpath," + os.path.dirname(blas), "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def reference_dir() -> str:
    """The reference checkout that build_ref.sh reads (it may not exist on this machine)."""
    out = subprocess.check_output(["bash", os.path.join(HERE, "build_ref.sh"), "--print-ref"])
    return out.decode().strip()


def build_reference() -> Optional[str]:
    """Build oracle/_ref from the reference sources when they are present (None otherwise)."""
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh"), "--if-present"])
    return REF_EXE if os.path.exists(REF_EXE) else None


class OracleCfg(ctypes.Structure):
    _fields_ = [("n_ind", ctypes.c_int), ("n_snp", ctypes.c_int), ("nsv", ctypes.c_int), ("nrhs", ctypes.c_int),
                ("power", ctypes.c_int), ("crit", ctypes.c_int), ("miter", ctypes.c_int), ("bsize", ctypes.c_int),
                ("tol", ctypes.c_double), ("threads", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.oracle_decode_stats.argtypes = [P, ctypes.c_int, ctypes.c_int, P, P, P]
        L.oracle_omega.argtypes = [ctypes.c_int, ctypes.c_int, P]
        L.oracle_pass.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int, P, P]
        L.oracle_pass.restype = ctypes.c_int
        L.oracle_synth_rows.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P,
                                        ctypes.c_int, P]
        L.oracle_solve.argtypes = [ctypes.POINTER(OracleCfg), P, P, P, P, ctypes.POINTER(ctypes.c_int), P, P]
        L.oracle_solve.restype = ctypes.c_int
        L.oracle_lut_row.argtypes = [ctypes.c_double, ctypes.c_double, P]
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def decode_stats(packed: np.ndarray, n_ind: int, want_codes: bool = False):
    """Per-SNP (avg, sd) as standardize() computes them, optionally the decoded codes."""
    packed = np.ascontiguousarray(packed, dtype=np.uint8)
    n_snp = packed.shape[0]
    avg = np.empty(n_snp)
    sd = np.empty(n_snp)
    codes = np.empty((n_snp, n_ind), dtype=np.uint8) if want_codes else None
    lib().oracle_decode_stats(_p(packed), n_ind, n_snp, _p(avg), _p(sd), _p(codes) if want_codes else None)
    return (avg, sd, codes) if want_codes else (avg, sd)


def lut(avg: float, sd: float) -> np.ndarray:
    out = np.empty(4)
    lib().oracle_lut_row(avg, sd, _p(out))
    return out


def omega(n_ind: int, k: int) -> np.ndarray:
    out = np.empty((n_ind, k))
    lib().oracle_omega(n_ind, k, _p(out))
    return out


def one_pass(packed: np.ndarray, n_ind: int, omega_: np.ndarray, bsize: int, npasses: int = 1, walls=None):
    """Z = X^T X Omega with the reference's blocked FP64 pass.

    Returns (Z, times) with times = [load/decode, X*Omega, X^T*Y, wall] seconds of the last
    of ``npasses`` passes (passes after the first use the per-SNP LUT cache)."""
    packed = np.ascontiguousarray(packed, dtype=np.uint8)
    om = np.ascontiguousarray(omega_, dtype=np.float64)
    z = np.empty_like(om)
    t = np.zeros(4)
    w = np.zeros(max(1, npasses))
    rc = lib().oracle_pass(_p(packed), n_ind, packed.shape[0], bsize, _p(om), om.shape[1], _p(z), npasses, _p(t),
                           _p(w))
    if walls is not None:
        walls.extend(w.tolist())
    if rc:
        raise MemoryError("oracle_pass allocation failed")
    return z, t


def synth_rows(cohort, s0: int, s1: int) -> np.ndarray:
    """Packed rows [s0, s1) of a distpca_gb300.synth cohort, generated in C."""
    out = np.empty((s1 - s0, (cohort.n_ind + 3) // 4), dtype=np.uint8)
    pop = np.ascontiguousarray(cohort.pop, dtype=np.uint8)
    miss = np.ascontiguousarray(cohort.miss_thr, dtype=np.uint32)
    thr = np.ascontiguousarray(cohort.snp_thr, dtype=np.uint32)
    lib().oracle_synth_rows(ctypes.c_uint64(cohort.key), cohort.n_ind, s0, s1, _p(pop), _p(miss), _p(thr),
                            cohort.n_pop, _p(out))
    return out


def set_threads(n: int) -> None:
    lib().oracle_set_threads(n)


def solve(packed: np.ndarray, n_ind: int, *, nsv: int, nrhs: int, power: int = 1, crit: int = 1,
          tol: float = 1e-3, miter: int = 100, bsize: int = 0, threads: int = 0,
          omega0: Optional[np.ndarray] = None) -> dict:
    """Run the restated solver; bsize >= n_snp selects the in-core variant."""
    packed = np.ascontiguousarray(packed, dtype=np.uint8)
    n_snp = packed.shape[0]
    om = omega(n_ind, nrhs) if omega0 is None else np.array(omega0, dtype=np.float64, order="C")
    cfg = OracleCfg(n_ind, n_snp, nsv, nrhs, power, crit, miter, bsize if bsize > 0 else n_snp, tol, threads)
    sigma = np.empty(nsv)
    u = np.empty((n_ind, nsv))
    its = ctypes.c_int(0)
    cv = np.full(max(miter, 1), np.nan)
    tm = np.zeros(6)
    rc = lib().oracle_solve(ctypes.byref(cfg), _p(packed), _p(om), _p(sigma), _p(u), ctypes.byref(its), _p(cv),
                            _p(tm))
    if rc:
        raise MemoryError("oracle_solve allocation failed")
    return {"sigma": sigma, "u": u, "omega": om, "its": its.value, "crit": cv[: its.value], "timers": tm}


def run_reference_cli(args, cwd: str, threads: int = 1, timeout: int = 600) -> str:
    """Run oracle/_ref/DistPCA.exe (the reference itself) and return stdout."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS=str(threads))
    return subprocess.run([REF_EXE] + list(args), cwd=cwd, env=env, capture_output=True, text=True,
                          timeout=timeout, check=True).stdout
