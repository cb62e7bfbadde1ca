"""Small cases of each kernel family, sized for one ncu capture, and a per-kernel breakdown of solves.

    python -m distpca_gb300.profcase incore     20,000 x 100,000 (0.5 GB packed, above L2 once
                                                transposed and split), nrhs 40, mixed: per-SNP
                                                statistics and the transpose at upload, two passes
                                                (X Omega, X^T Y), then a two-iteration solve
                                                (Cholesky QR, Jacobi eigensolver, criterion)
    python -m distpca_gb300.profcase small      1,000 x 100,000, nrhs 20, mixed: two passes and a
                                                two-iteration solve (X Omega's short-K shape)
    python -m distpca_gb300.profcase windows    256 windows over 2,000 individuals, nrhs 8: the
                                                batched windows' passes, QR and Rayleigh-Ritz kernels
    python -m distpca_gb300.profcase breakdown  per-kernel device time (the handle's kernel clock)
                                                of whole converged solves: the 1,000 x 100,000
                                                cohort (nsv 10, nrhs 20, power 4, tol 1e-6) and
                                                two serving-size jobs, mixed and FP64
    python -m distpca_gb300.profcase qr         the device QR of random panels at four shapes, as one
                                                launch and as separate kernels (for a launch list)
    python -m distpca_gb300.profcase passes     per-launch device time of a mixed pass's kernels at
                                                four serving-size shapes
    python -m distpca_gb300.profcase stream     the 512 jobs of the serving stream (serve_stream,
                                                seed 0) solved one at a time, mixed: wall time,
                                                then per-kernel device time summed over the jobs
                                                and split by job size

Each case holds well under 1 GB on the device and launches each kernel a handful of times, so that
an ncu capture of one launch (`-k <kernel> -c 1`) ends by itself in a minute or two.
"""
from __future__ import annotations

import json
import sys
import time

import numpy as np

from . import api as D
from . import synth


def incore() -> None:
    n_ind, n_snp, k = 20000, 100000, 40
    c = synth.config_cohort("incore50k", n_snp=n_snp, n_ind=n_ind)
    with D.Handle(n_ind, n_snp, k, precision="mixed") as h:
        h.synth_fill(c)
        om = D.start_block(n_ind, k)
        h.set_omega(om)
        h.pass_()
        h.pass_()
        h.synchronize()
        r = h.solve(om, nsv=20, power=2, crit=1, tol=-1, miter=2, bsize=10000)
    print("incore ok, iterations", r["its"])


def small() -> None:
    """1,000 individuals x 100,000 SNPs, nrhs 20, mixed: two passes and a two-iteration solve (the
    short-K shape of X Omega: 16 K-blocks per row tile)."""
    n_ind, n_snp, k = 1000, 100000, 20
    c = synth.make_cohort(n_ind, n_snp, n_pop=5, fst=0.05, missing=0.01, seed=0)
    with D.Handle(n_ind, n_snp, k, precision="mixed") as h:
        h.synth_fill(c)
        om = D.start_block(n_ind, k)
        h.set_omega(om)
        h.pass_()
        h.pass_()
        h.synchronize()
        r = h.solve(om, nsv=10, power=4, crit=1, tol=-1, miter=2, bsize=n_snp)
    print("small ok, iterations", r["its"])


def windows() -> None:
    widths = synth.window_widths(256, seed=0)
    cw = synth.make_cohort(2000, int(widths.sum()), n_pop=4, fst=0.05, missing=0.01, seed=4)
    with D.Windows(2000, widths, 8) as w:
        w.synth_fill(cw)
        w.solve(nsv=2, power=3, miter=2, want_u=False)
    print("windows ok")


BREAKDOWN = [
    # name, n_ind, n_snp, nrhs, nsv, power, tol, bsize, cohort
    ("1k_x_100k", 1000, 100000, 20, 10, 4, 1e-6, 10000,
     dict(n_pop=5, pop_sizes=[200] * 5, fst=0.05, p_range=(0.05, 0.5), missing=0.01, seed=0)),
    ("job_4765_x_134387", 4765, 134387, 40, 20, 4, 1e-3, 134387, dict(n_pop=4, fst=0.05, missing=0.01, seed=3)),
    ("job_2813_x_37351", 2813, 37351, 10, 5, 4, 1e-3, 37351, dict(n_pop=3, fst=0.05, missing=0.01, seed=4)),
]


def breakdown() -> None:
    for name, n, m, k, nsv, power, tol, bsize, ckw in BREAKDOWN:
        c = synth.make_cohort(n, m, **ckw)
        for prec in ("mixed", "fp64"):
            with D.Handle(n, m, k, precision=prec) as h:
                h.synth_fill(c)
                om = D.start_block(n, k)
                h.solve(om, nsv=nsv, power=power, crit=1, tol=tol, miter=2, bsize=bsize)
                h.reset_kernel_times(True)
                t0 = time.perf_counter()
                r = h.solve(om, nsv=nsv, power=power, crit=1, tol=tol, miter=100, bsize=bsize)
                wall = time.perf_counter() - t0
                kt = h.kernel_times()
            tot = sum(v["ms"] for v in kt.values())
            per = {a: [round(v["ms"], 3), v["launches"]] for a, v in sorted(kt.items(), key=lambda x: -x[1]["ms"])}
            print(json.dumps({"case": name, "precision": prec, "its": r["its"], "wall_ms": round(wall * 1e3, 2),
                              "kernel_ms_total": round(tot, 2), "per_kernel_ms_launches": per}), flush=True)


PASS_SHAPES = [(1000, 100000, 20), (2813, 37351, 10), (4765, 134387, 40), (20000, 100000, 40)]
QR_SHAPES = [(1000, 10), (1000, 20), (4765, 40), (20000, 40)]


def qr() -> None:
    """The device QR of random panels at serving-size shapes, twice as one cooperative launch and
    twice as separate kernels (for a per-kernel launch list); prints max |Q^T Q - I|."""
    rng = np.random.default_rng(0)
    for n, k in QR_SHAPES:
        a = rng.standard_normal((n, k))
        for separate in (False, True):
            for _ in range(2):
                q = D.qr_device(a, separate=separate)
        print(n, k, float(np.abs(q.T @ q - np.eye(k)).max()))


def passes() -> None:
    """Per-launch device time of a mixed pass's kernels at serving-size shapes: 3 warm-up passes,
    then 20 under the per-launch clock."""
    out = {}
    for n, m, k in PASS_SHAPES:
        c = synth.make_cohort(n, m, n_pop=4, fst=0.05, missing=0.01, seed=1)
        with D.Handle(n, m, k, precision="mixed") as h:
            h.synth_fill(c)
            h.set_omega(D.start_block(n, k))
            for _ in range(3):
                h.pass_()
            h.synchronize()
            h.reset_kernel_times(True)
            for _ in range(20):
                h.pass_()
            h.synchronize()
            kt = h.kernel_times()
        out[f"{n}x{m}_nrhs{k}"] = {a: round(v["ms"] / v["launches"] * 1e3, 1) for a, v in kt.items() if v["launches"]}
    print(json.dumps({"us_per_launch": out}))


def _kernel_family(name: str) -> str:
    if name in ("mixed_xw", "mixed_xty", "mixed_reduce", "split_omega", "split_bop"):
        return "products"
    if name.startswith("qr"):
        return "qr"
    if name in ("atb", "sym_eig", "apply_w"):
        return "rayleigh_ritz"
    if name in ("synth_fill", "snp_stats", "transpose_packed"):
        return "setup"
    return "other"


def stream() -> None:
    jobs = synth.serve_stream(512, 50.0, seed=0)
    cohorts = [synth.serve_cohort(j) for j in jobs]

    def one(j, c, clock):
        t0 = time.perf_counter()
        with D.Handle(j["n_ind"], j["n_snp"], j["nrhs"], precision="mixed") as h:
            if clock:
                h.reset_kernel_times(True)
            h.synth_fill(c)
            r = h.solve(D.start_block(j["n_ind"], j["nrhs"]), nsv=j["nsv"], power=j["power"], bsize=j["n_snp"])
            kt = h.kernel_times() if clock else {}
        return time.perf_counter() - t0, r, kt

    one(jobs[0], cohorts[0], False)  # warm-up: the library's one-time device setup
    walls = np.array([one(j, c, False)[0] for j, c in zip(jobs, cohorts)])
    print(json.dumps({"jobs": len(jobs), "one_at_a_time_s": round(float(walls.sum()), 3),
                      "jobs_per_s": round(len(jobs) / float(walls.sum()), 2)}), flush=True)
    geno = np.array([j["n_ind"] * j["n_snp"] for j in jobs], dtype=np.float64)
    edges = np.quantile(geno, [0.25, 0.5, 0.75])
    per_kernel: dict = {}
    fam = np.zeros((4, 5))  # size quartile x (products, qr, rayleigh_ritz, setup, other)
    names = ["products", "qr", "rayleigh_ritz", "setup", "other"]
    passes = 0
    for i, (j, c) in enumerate(zip(jobs, cohorts)):
        _, r, kt = one(j, c, True)
        passes += int(r["passes"])
        q = int(np.searchsorted(edges, geno[i], side="right"))
        for a, v in kt.items():
            e = per_kernel.setdefault(a, [0.0, 0])
            e[0] += v["ms"]
            e[1] += v["launches"]
            fam[q, names.index(_kernel_family(a))] += v["ms"]
    tot = sum(v[0] for v in per_kernel.values())
    print(json.dumps({"kernel_ms_total": round(tot, 1), "passes": passes,
                      "per_kernel_ms_launches": {a: [round(v[0], 1), v[1]] for a, v in
                                                 sorted(per_kernel.items(), key=lambda x: -x[1][0])}}), flush=True)
    for q in range(4):
        sel = np.searchsorted(edges, geno, side="right") == q
        print(json.dumps({"size_quartile": q, "jobs": int(sel.sum()),
                          "genotypes": [float(geno[sel].min()), float(geno[sel].max())],
                          "one_at_a_time_s": round(float(walls[sel].sum()), 3),
                          "kernel_ms": {n: round(float(fam[q, f]), 1) for f, n in enumerate(names)}}), flush=True)


CASES = {"incore": incore, "small": small, "windows": windows, "breakdown": breakdown, "stream": stream,
         "passes": passes, "qr": qr}


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    names = argv or ["incore", "windows"]
    for a in names:
        if a not in CASES:
            print(f"unknown case {a!r}; cases: {', '.join(CASES)}", file=sys.stderr)
            return 2
    np.set_printoptions(precision=4)
    for a in names:
        CASES[a]()
    return 0


if __name__ == "__main__":
    sys.exit(main())
