"""Locate the LP64 OpenBLAS that ships inside the scipy wheel.

Test infrastructure: the CPU oracle (the reference build in oracle/_ref and the
C restatement in oracle/dpca_oracle.c) links this library for its dense
BLAS/LAPACK calls, the same way the reference links MKL or OpenBLAS.
Prints the absolute path of the shared object, or exits 1.
"""
import glob
import os
import sys


def find():
    """(path, ilp64): scipy's LP64 library, else numpy's ILP64 one."""
    import numpy
    try:
        import scipy

        base = os.path.dirname(os.path.dirname(os.path.abspath(scipy.__file__)))
        cands = sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
        cands = [c for c in cands if "64_" not in os.path.basename(c)]
        if cands:
            return cands[0], False
    except ImportError:
        pass
    base = os.path.dirname(os.path.dirname(os.path.abspath(numpy.__file__)))
    cands = sorted(glob.glob(os.path.join(base, "numpy.libs", "libscipy_openblas64_*.so*")))
    if cands:
        return cands[0], True
    raise FileNotFoundError("no bundled OpenBLAS in the scipy or numpy wheels")


if __name__ == "__main__":
    try:
        path, ilp64 = find()
        if ilp64:
            print("ILP64 build found; the reference oracle needs LP64", file=sys.stderr)
            sys.exit(1)
        print(path)
    except Exception as exc:  # pragma: no cover - reported to the build script
        print(f"find_openblas: {exc}", file=sys.stderr)
        sys.exit(1)
