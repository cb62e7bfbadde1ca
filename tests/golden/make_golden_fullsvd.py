"""Golden vectors of the reference's -fullSVD accuracy check (distpca.cpp:449-635) on the
`small` fixture: the reference build (oracle/_ref/DistPCA.exe, its own LAPACKE_dgesvd through
the oracle's OpenBLAS shim) run with -fullSVD 1 -fwrite 1.  Writes small_fullsvd.npz (true
singular values, |true left singular vectors|, cosine values, the approximate sigma) and the head
of each text file, for the file-format test.  Run from the repository root:

    python tests/golden/make_golden_fullsvd.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402

FLAGS = ["-nsv", "5", "-nrhs", "10", "-power", "2", "-crit", "1", "-tol", "1e-6", "-bsize", "2500"]
FILES = ("realSingularValues", "realLeftSingularVectors", "singvecs_accuracy", "cosineValues", "singularValues")


def main() -> None:
    if not os.path.exists(O.REF_EXE):
        O.build_reference()
    with tempfile.TemporaryDirectory() as td:
        pref = os.path.join(td, "r")
        args = ["-bfile", os.path.join(HERE, "small"), "-fwrite", "1", "-verbose", "2", "-fullSVD", "1",
                "-prefix", pref] + FLAGS
        out = O.run_reference_cli(args, cwd=td, threads=1)
        true_sigma = np.loadtxt(pref + "_realSingularValues.txt", ndmin=1)
        true_u = np.loadtxt(pref + "_realLeftSingularVectors.txt", ndmin=2)
        cosines = np.loadtxt(pref + "_cosineValues.txt", ndmin=1)
        sigma = np.loadtxt(pref + "_singularValues.txt", ndmin=1)
        for name in FILES[:4]:
            with open(f"{pref}_{name}.txt") as f, open(os.path.join(HERE, f"small_fullsvd_ref_{name}.txt"), "w") as g:
                g.writelines(f.readlines()[:6])
        rel = [ln for ln in out.splitlines() if ln.startswith("RelError Sigma")]
    np.savez_compressed(os.path.join(HERE, "small_fullsvd.npz"), true_sigma=true_sigma, true_u_abs=np.abs(true_u),
                        cosines=cosines, sigma=sigma, flags=np.array(FLAGS), relerr_lines=np.array(rel))
    print("true sigma", true_sigma, "cosines", cosines)


if __name__ == "__main__":
    main()
