"""Regenerate the golden fixtures from the reference itself.

Writes small seeded PLINK filesets (tiny, small, wide) into tests/golden/ and
records what the UNMODIFIED reference computes on them, using the binaries
that oracle/build_ref.sh builds from the reference sources:
  - ref_harness stats: per-SNP avg/sd of standardize() after decode_plink_sse2,
    plus checksums of the decoded codes and standardized rows;
  - ref_harness omega: the start block of distpca.cpp:389-394;
  - DistPCA.exe runs (1 BLAS thread, -fwrite 1, -verbose 2): singular values,
    left singular vectors, iteration count and the per-iteration criterion lines.
Everything lands in golden.npz and *_ref_*.txt next to this script.

Run from the repository root:  python tests/golden/make_golden.py
Needs the reference checkout that oracle/build_ref.sh reads (DPCA_REFERENCE overrides it).
"""
from __future__ import annotations

import hashlib
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from distpca_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

RUNS = {
    # name: (fileset, flags)
    "small_ooc": ("small", ["-nsv", "5", "-nrhs", "10", "-power", "2", "-crit", "1", "-tol", "1e-6", "-bsize", "400"]),
    "small_incore": ("small", ["-nsv", "5", "-nrhs", "10", "-power", "2", "-crit", "1", "-tol", "1e-6",
                               "-bsize", "2500"]),
    "small_mev": ("small", ["-nsv", "4", "-nrhs", "8", "-power", "1", "-crit", "2", "-tol", "1e-4", "-bsize", "1000"]),
    "small_trace": ("small", ["-nsv", "6", "-nrhs", "12", "-crit", "0", "-tol", "1e-9", "-miter", "7",
                              "-bsize", "333"]),
    "small_fixed3": ("small", ["-nsv", "5", "-nrhs", "10", "-crit", "1", "-tol", "-1", "-miter", "3",
                               "-bsize", "777"]),
    "tiny_edges": ("tiny", ["-nsv", "3", "-nrhs", "6", "-bsize", "50", "-crit", "1", "-tol", "1e-4"]),
    "tiny_clamp": ("tiny", ["-nsv", "40", "-nrhs", "5", "-bsize", "64", "-crit", "1", "-tol", "1e-3",
                            "-miter", "4"]),
    "wide_mev": ("wide", ["-nsv", "10", "-nrhs", "20", "-power", "3", "-bsize", "100", "-crit", "2",
                          "-tol", "1e-5"]),
}


def tiny_packed() -> np.ndarray:
    c = synth.make_cohort(37, 300, n_pop=3, fst=0.1, missing=0.05, seed=11)
    codes = synth.genotype_codes(c, 0, 300)
    codes[0, :] = 0b00            # monomorphic hom A1
    codes[1, :] = 0b01            # all missing
    codes[2, :] = 0b11            # monomorphic hom A2
    codes[3, :] = 0b00
    codes[3, 17] = 0b10           # single het
    codes[4, :] = 0b01
    codes[4, 5] = 0b11            # one observed genotype
    codes[5, :] = np.arange(37) % 4  # every code
    codes[6, :] = 0b10            # all het: p = 0.5
    packed = synth.pack_codes(codes)
    # non-zero padding bits in the last byte of some rows (ignored by the decoder)
    packed[7:20, -1] |= 0b11 << 2 * (37 % 4)
    return packed


def filesets():
    out = {}
    out["tiny"] = (37, tiny_packed())
    c = synth.make_cohort(203, 2500, n_pop=4, dirichlet=True, fst=0.05, p_range=(0.02, 0.5), missing=0.02, seed=5)
    out["small"] = (203, synth.pack_rows(c))
    c = synth.make_cohort(1001, 800, n_pop=5, fst=0.08, missing=0.01, seed=9)
    out["wide"] = (1001, synth.pack_rows(c))
    return out


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def parse_run(stdout: str, prefix: str, power: int):
    crit_lines = [ln for ln in stdout.splitlines() if ln.startswith("Iteration ")]
    # -verbose 2 prints one criterion line per iteration ii >= 1 and breaks right after the
    # converged one, so the iteration count is the number of lines plus one
    its = len(crit_lines) + 1
    m = re.search(r"fetched from the memory: (\d+)", stdout)
    if m and int(m.group(1)) != its * (power + 1):
        raise RuntimeError(f"pass count {m.group(1)} disagrees with {its} iterations")
    sv = np.loadtxt(prefix + "_singularValues.txt", ndmin=1)
    with open(prefix + "_leftSingularVectors.txt") as f:
        lines = f.read().splitlines()
    u = np.array([[float(x) for x in ln.split("\t")[1:]] for ln in lines[1:]])
    return its, crit_lines, sv, u


def main() -> None:
    if not os.path.exists(O.REF_EXE):
        O.build_reference()
    fs = filesets()
    data = {}
    for name, (n_ind, packed) in fs.items():
        prefix = os.path.join(HERE, name)
        synth.write_plink(prefix, packed, n_ind)
        n_snp = packed.shape[0]
        with tempfile.TemporaryDirectory() as td:
            outp = os.path.join(td, "stats.bin")
            subprocess.check_call([O.REF_HARNESS, "stats", prefix, str(n_ind), str(n_snp), outp])
            raw = np.fromfile(outp, dtype=np.uint8)
        rec = 16 + 8 * n_ind + n_ind
        raw = raw.reshape(n_snp, rec)
        avg = raw[:, 0:8].copy().view(np.float64).ravel()
        sd = raw[:, 8:16].copy().view(np.float64).ravel()
        norm = raw[:, 16:16 + 8 * n_ind].copy().view(np.float64).reshape(n_snp, n_ind)
        dec = raw[:, 16 + 8 * n_ind:].copy()
        data[f"{name}_avg"] = avg
        data[f"{name}_sd"] = sd
        data[f"{name}_norm_sha"] = np.array(sha(norm))
        data[f"{name}_dec_sha"] = np.array(sha(dec))
        data[f"{name}_norm_rows"] = norm[:8]
        data[f"{name}_dec_rows"] = dec[:8]
    for (n, k) in [(37, 6), (203, 10), (1001, 20), (50000, 2)]:
        with tempfile.TemporaryDirectory() as td:
            outp = os.path.join(td, "om.bin")
            subprocess.check_call([O.REF_HARNESS, "omega", str(n), str(k), outp])
            om = np.fromfile(outp).reshape(n, k)
        data[f"omega_{n}x{k}_sha"] = np.array(sha(om))
        data[f"omega_{n}x{k}_head"] = om[:4]
        if n > 46340:  # rows around the 32-bit seed wrap of jj*M+kk
            data[f"omega_{n}x{k}_wrap"] = om[42945:42955]
            data[f"omega_{n}x{k}_tail"] = om[-3:]
        elif n * k <= 20000:
            data[f"omega_{n}x{k}"] = om
    for run, (fset, flags) in RUNS.items():
        with tempfile.TemporaryDirectory() as td:
            pref = os.path.join(td, "r")
            args = ["-bfile", os.path.join(HERE, fset), "-fwrite", "1", "-verbose", "2", "-prefix", pref] + flags
            out = O.run_reference_cli(args, cwd=td, threads=1)
            power = int(flags[flags.index("-power") + 1]) if "-power" in flags else 1
            its, crit_lines, sv, u = parse_run(out, pref, power)
            for suffix in ("singularValues", "leftSingularVectors"):
                with open(f"{pref}_{suffix}.txt") as f, open(os.path.join(HERE, f"{run}_ref_{suffix}.txt"), "w") as g:
                    g.writelines(f.readlines()[:12])  # the text formats; values live in golden.npz
        data[f"run_{run}_its"] = np.array(its)
        data[f"run_{run}_sigma"] = sv
        data[f"run_{run}_u"] = u
        data[f"run_{run}_crit"] = np.array(crit_lines)
        data[f"run_{run}_flags"] = np.array(flags)
        data[f"run_{run}_fileset"] = np.array(fset)
        print(run, "its", its, "sigma", sv[:3])
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **data)
    print("wrote", os.path.join(HERE, "golden.npz"))


if __name__ == "__main__":
    main()
