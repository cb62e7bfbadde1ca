"""Golden results of the reference at the two workloads its users run first.

  cfg1   the 1,000 x 100,000 cohort of the CPU-parity workload (seeded Balding-Nichols: K = 5
         populations of 200, Fst 0.05, p ~ U(0.05, 0.5), 1% missing, seed 0) with nsv 10,
         nrhs 20, power 4, tol 1e-6, bsize 10,000 -- a whole converged PCA -- and the same
         matrix at a fixed 4 iterations (-crit 1 -tol -1) and under the published runs'
         -crit 2 -tol 1e-3;
  hgdp   the reference's own example fileset (example/hgdp.qc.pruned, 942 x 133,594) with the
         flags of its published log (-nsv 20 -nrhs 40 -crit 2 -tol 1e-3 -bsize 100: 22 passes,
         example/hgdp.qc.pruned.log:40), and at a fixed 3 iterations.

Every run is the UNMODIFIED reference (oracle/_ref/DistPCA.exe, built by oracle/build_ref.sh)
on one BLAS thread.  The cfg1 matrix is not stored: tests rebuild it from the seed and check
its SHA-256 against the one recorded here.  The HGDP fileset belongs to the reference checkout
and is not copied: tests read it from $DPCA_HGDP_BFILE and skip when that is unset, after
checking the .bed's SHA-256.  Outputs: tests/golden/configs.npz.

Run from the repository root:  python tests/golden/make_golden_configs.py   (~10 min)
"""
from __future__ import annotations

import hashlib
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from distpca_gb300 import synth  # noqa: E402
from make_golden import parse_run  # noqa: E402
from oracle import oracle as O  # noqa: E402

CFG1 = dict(n_ind=1000, n_snp=100_000, n_pop=5, pop_sizes=[200] * 5, fst=0.05, p_range=(0.05, 0.5),
            missing=0.01, seed=0)

RUNS = {
    "cfg1": ("cfg1", ["-nsv", "10", "-nrhs", "20", "-power", "4", "-tol", "1e-6", "-bsize", "10000"]),
    "cfg1_fixed4": ("cfg1", ["-nsv", "10", "-nrhs", "20", "-power", "4", "-crit", "1", "-tol", "-1", "-miter", "4",
                             "-bsize", "10000"]),
    "cfg1_mev": ("cfg1", ["-nsv", "10", "-nrhs", "20", "-power", "4", "-crit", "2", "-tol", "1e-3",
                          "-bsize", "10000"]),
    "hgdp": ("hgdp", ["-nsv", "20", "-nrhs", "40", "-crit", "2", "-tol", "1e-3", "-bsize", "100"]),
    "hgdp_fixed3": ("hgdp", ["-nsv", "20", "-nrhs", "40", "-crit", "1", "-tol", "-1", "-miter", "3",
                             "-bsize", "100"]),
}


def cfg1_cohort():
    kw = dict(CFG1)
    n_ind, n_snp = kw.pop("n_ind"), kw.pop("n_snp")
    return synth.make_cohort(n_ind, n_snp, **kw)


def sha_file(path: str) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for chunk in iter(lambda: f.read(1 << 20), b""):
            h.update(chunk)
    return h.hexdigest()


def main() -> None:
    if not os.path.exists(O.REF_EXE):
        O.build_reference()
    work = tempfile.mkdtemp(prefix="dpca_golden_")
    data = {}
    try:
        c = cfg1_cohort()
        packed = O.synth_rows(c, 0, c.n_snp)
        prefixes = {"cfg1": os.path.join(work, "cfg1"),
                    "hgdp": os.path.join(O.reference_dir(), "example", "hgdp.qc.pruned")}
        synth.write_plink(prefixes["cfg1"], packed, c.n_ind)
        data["cfg1_packed_sha"] = np.array(hashlib.sha256(packed.tobytes()).hexdigest())
        data["hgdp_bed_sha"] = np.array(sha_file(prefixes["hgdp"] + ".bed"))
        for run, (fset, flags) in RUNS.items():
            pref = os.path.join(work, run)
            args = ["-bfile", prefixes[fset], "-fwrite", "1", "-verbose", "2", "-prefix", pref] + flags
            out = O.run_reference_cli(args, cwd=work, threads=1, timeout=3600)
            power = int(flags[flags.index("-power") + 1]) if "-power" in flags else 1
            its, crit_lines, sv, u = parse_run(out, pref, power)
            data[f"run_{run}_its"] = np.array(its)
            data[f"run_{run}_sigma"] = sv
            data[f"run_{run}_u"] = u
            data[f"run_{run}_crit"] = np.array(crit_lines)
            data[f"run_{run}_flags"] = np.array(flags)
            data[f"run_{run}_fileset"] = np.array(fset)
            print(run, "its", its, "passes", its * (power + 1), "sigma", sv[:3], flush=True)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    np.savez_compressed(os.path.join(HERE, "configs.npz"), **data)
    print("wrote", os.path.join(HERE, "configs.npz"))


if __name__ == "__main__":
    main()
