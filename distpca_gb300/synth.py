"""Seeded Balding-Nichols cohorts in PLINK SNP-major .bed format.

Population structure (tables) is drawn with numpy from one seed; genotypes
are then a pure function of (seed, snp, individual) through a 64-bit
counter hash, so any block of SNPs can be produced independently and the
CUDA fill kernel (``dpca_synth_fill`` in libdpca) writes the very same bytes
as :func:`pack_rows` here.

Model: ancestral allele frequency p per SNP; per population k,
p_k ~ Beta(p(1-F)/F, (1-p)(1-F)/F); genotype g ~ Binomial(2, p_k) drawn as
two Bernoulli alleles; missing entries per a per-individual rate.
Encoding (PLINK 1 SNP-major): g=0 -> 00, g=1 -> 10, g=2 -> 11,
missing -> 01; four samples per byte, first sample in the low bits; header
0x6C 0x1B 0x01.
"""
from __future__ import annotations

import dataclasses
import os
from typing import Optional, Sequence

import numpy as np

MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)
GOLD = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)
MISS_SALT = np.uint64(0xD6E8FEB86659FD93)
BED_MAGIC = bytes([0x6C, 0x1B, 0x01])


def _fmix(z: np.ndarray) -> np.ndarray:
    """splitmix64 output function (wrapping uint64 arithmetic)."""
    z = (z ^ (z >> np.uint64(30))) * M1
    z = (z ^ (z >> np.uint64(27))) * M2
    return z ^ (z >> np.uint64(31))


def seed_key(seed: int) -> int:
    with np.errstate(over="ignore"):
        return int(_fmix(np.array([np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + GOLD], dtype=np.uint64))[0])


@dataclasses.dataclass
class Cohort:
    """Tables that fully determine a synthetic cohort."""

    n_ind: int
    n_snp: int
    seed: int
    pop: np.ndarray        # uint8 [n_ind] population of each individual
    miss_thr: np.ndarray   # uint32 [n_ind] missing if hash32 < thr
    snp_thr: np.ndarray    # uint32 [n_snp, K] allele draw is 1 if hash32 < thr
    n_pop: int

    @property
    def key(self) -> int:
        return seed_key(self.seed)

    @property
    def bytes_per_snp(self) -> int:
        return (self.n_ind + 3) // 4


def make_cohort(
    n_ind: int,
    n_snp: int,
    *,
    n_pop: int = 5,
    pop_sizes: Optional[Sequence[int]] = None,
    dirichlet: bool = False,
    fst: float = 0.05,
    p_range: tuple = (0.05, 0.5),
    p_beta: Optional[tuple] = None,
    p_clip: tuple = (0.0, 1.0),
    missing: float = 0.01,
    heavy_frac: float = 0.0,
    heavy_rate: float = 0.0,
    seed: int = 0,
) -> Cohort:
    """Draw the population tables of a Balding-Nichols cohort.

    ``pop_sizes`` fixes the population sizes; otherwise sizes are equal, or
    Dirichlet(1) proportions when ``dirichlet``.  Ancestral frequencies are
    U(p_range) unless ``p_beta=(a, b)`` (then Beta(a, b) clipped to
    ``p_clip``).  ``missing`` is an i.i.d. per-entry rate; with
    ``heavy_frac > 0`` a random ``heavy_frac`` of the samples get
    ``heavy_rate`` and the rest ``missing``.
    """
    rng = np.random.default_rng(seed)
    if pop_sizes is None:
        if dirichlet:
            prop = rng.dirichlet(np.ones(n_pop))
            sizes = np.floor(prop * n_ind).astype(np.int64)
            sizes[np.argmax(sizes)] += n_ind - sizes.sum()
        else:
            sizes = np.full(n_pop, n_ind // n_pop, dtype=np.int64)
            sizes[: n_ind - sizes.sum()] += 1
    else:
        sizes = np.asarray(pop_sizes, dtype=np.int64)
        if sizes.sum() != n_ind:
            raise ValueError("pop_sizes must sum to n_ind")
    pop = np.repeat(np.arange(len(sizes), dtype=np.uint8), sizes)
    if p_beta is None:
        p = rng.uniform(p_range[0], p_range[1], size=n_snp)
    else:
        p = np.clip(rng.beta(p_beta[0], p_beta[1], size=n_snp), p_clip[0], p_clip[1])
    a = p[:, None] * (1.0 - fst) / fst
    b = (1.0 - p[:, None]) * (1.0 - fst) / fst
    pk = rng.beta(np.broadcast_to(a, (n_snp, len(sizes))), np.broadcast_to(b, (n_snp, len(sizes))))
    snp_thr = np.minimum(np.floor(pk * 4294967296.0), 4294967295.0).astype(np.uint32)
    rate = np.full(n_ind, missing, dtype=np.float64)
    if heavy_frac > 0:
        heavy = rng.choice(n_ind, size=int(round(heavy_frac * n_ind)), replace=False)
        rate[heavy] = heavy_rate
    miss_thr = np.minimum(np.floor(rate * 4294967296.0), 4294967295.0).astype(np.uint32)
    return Cohort(n_ind, n_snp, seed, pop, miss_thr, np.ascontiguousarray(snp_thr), len(sizes))


def genotype_codes(c: Cohort, s0: int, s1: int) -> np.ndarray:
    """2-bit PLINK codes (uint8 0..3) of SNPs [s0, s1) x all individuals."""
    key = np.uint64(c.key)
    s = np.arange(s0, s1, dtype=np.uint64)[:, None]
    i = np.arange(c.n_ind, dtype=np.uint64)[None, :]
    with np.errstate(over="ignore"):
        x = ((s << np.uint64(32)) | i) ^ key
        h = _fmix(x + GOLD)
        hm = _fmix(x ^ MISS_SALT)
    thr = c.snp_thr[s0:s1][:, c.pop]  # [rows, n_ind]
    a1 = (h & np.uint64(0xFFFFFFFF)).astype(np.uint32) < thr
    a2 = (h >> np.uint64(32)).astype(np.uint32) < thr
    g = a1.astype(np.uint8) + a2.astype(np.uint8)
    miss = (hm & np.uint64(0xFFFFFFFF)).astype(np.uint32) < c.miss_thr[None, :]
    # g=0 -> 0b00, g=1 -> 0b10, g=2 -> 0b11, missing -> 0b01
    code = np.array([0, 2, 3], dtype=np.uint8)[g]
    code[miss] = 1
    return code


def pack_codes(codes: np.ndarray) -> np.ndarray:
    """Pack [rows, n_ind] 2-bit codes into [rows, ceil(n_ind/4)] bytes (pad = 00)."""
    rows, n = codes.shape
    nb = (n + 3) // 4
    pad = np.zeros((rows, nb * 4), dtype=np.uint8)
    pad[:, :n] = codes
    q = pad.reshape(rows, nb, 4)
    return (q[:, :, 0] | (q[:, :, 1] << 2) | (q[:, :, 2] << 4) | (q[:, :, 3] << 6)).astype(np.uint8)


def pack_rows(c: Cohort, s0: int = 0, s1: Optional[int] = None, chunk: int = 4096) -> np.ndarray:
    """Packed .bed rows (without header) of SNPs [s0, s1)."""
    s1 = c.n_snp if s1 is None else s1
    out = np.empty((s1 - s0, c.bytes_per_snp), dtype=np.uint8)
    step = max(1, min(chunk, (1 << 24) // max(1, c.n_ind)))
    for a in range(s0, s1, step):
        b = min(s1, a + step)
        out[a - s0 : b - s0] = pack_codes(genotype_codes(c, a, b))
    return out


def unpack_codes(packed: np.ndarray, n_ind: int) -> np.ndarray:
    """Inverse of :func:`pack_codes` (drops the padding codes)."""
    q = np.stack([(packed >> (2 * j)) & 3 for j in range(4)], axis=-1)
    return q.reshape(packed.shape[0], -1)[:, :n_ind].astype(np.uint8)


def write_plink(prefix: str, packed: np.ndarray, n_ind: int, *, iids: Optional[Sequence[str]] = None) -> None:
    """Write prefix.bed/.bim/.fam for packed SNP-major rows."""
    n_snp = packed.shape[0]
    os.makedirs(os.path.dirname(os.path.abspath(prefix)), exist_ok=True)
    with open(prefix + ".bed", "wb") as f:
        f.write(BED_MAGIC)
        f.write(np.ascontiguousarray(packed).tobytes())
    with open(prefix + ".bim", "w") as f:
        for s in range(n_snp):
            f.write(f"1\tsnp{s}\t0\t{s + 1}\tA\tG\n")
    if iids is None:
        iids = [f"IND{i}" for i in range(n_ind)]
    with open(prefix + ".fam", "w") as f:
        for i, iid in enumerate(iids):
            f.write(f"FAM{i}\t{iid}\t0\t0\t0\t-9\n")


def read_bed(prefix: str, n_ind: int, n_snp: int) -> np.ndarray:
    """Packed rows of prefix.bed (header skipped, not validated)."""
    nb = (n_ind + 3) // 4
    raw = np.fromfile(prefix + ".bed", dtype=np.uint8, count=3 + nb * n_snp)
    return raw[3:].reshape(n_snp, nb)


# Named cohorts with the shapes and distributions of the benchmark configurations.
def config_cohort(name: str, n_snp: Optional[int] = None, n_ind: Optional[int] = None) -> Cohort:
    if name == "cpu1k":  # 1,000 x 100,000, K=5 x 200, Fst 0.05, p~U(.05,.5), 1% missing, seed 0
        return make_cohort(n_ind or 1000, n_snp or 100_000, n_pop=5, fst=0.05, p_range=(0.05, 0.5),
                           missing=0.01, seed=0)
    if name == "incore50k":  # 50,000 x 1,000,000, K=8 Dirichlet(1), Fst 0.02, p~U(.01,.5), 2% missing
        return make_cohort(n_ind or 50_000, n_snp or 1_000_000, n_pop=8, dirichlet=True, fst=0.02,
                           p_range=(0.01, 0.5), missing=0.02, seed=2)
    if name == "stream500k":  # 500,000 x 2,000,000, K=10, Fst 0.01, Beta(.5,2) clipped, 5% in 10% of samples
        return make_cohort(n_ind or 500_000, n_snp or 2_000_000, n_pop=10, fst=0.01, p_beta=(0.5, 2.0),
                           p_clip=(0.005, 0.5), missing=0.0, heavy_frac=0.1, heavy_rate=0.5, seed=3)
    raise KeyError(name)


def serve_stream(n_jobs: int = 512, rate: float = 50.0, seed: int = 0) -> list:
    """A mixed-size PCA job stream: Poisson arrivals at `rate` jobs/s.

    Per job, seeded independently: n_ind log-uniform in [500, 20,000], n_snp log-uniform in
    [10,000, 500,000], nsv uniform in {5, 10, 20}, nrhs = 2 nsv, power 4, a Balding-Nichols
    cohort with K uniform in 2..8 populations, Fst uniform in [0.01, 0.1] and 0-3% missing.
    Returns dicts with the arrival time `t` (s), the sizes, the run flags and the cohort
    parameters (make_cohort draws the tables)."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n_jobs))
    jobs = []
    for j in range(n_jobs):
        n = int(round(float(np.exp(rng.uniform(np.log(500), np.log(20000))))))
        m = int(round(float(np.exp(rng.uniform(np.log(1e4), np.log(5e5))))))
        nsv = int(rng.choice([5, 10, 20]))
        jobs.append(dict(t=float(arrivals[j]), n_ind=n, n_snp=m, nsv=nsv, nrhs=2 * nsv, power=4,
                         n_pop=int(rng.integers(2, 9)), fst=float(rng.uniform(0.01, 0.1)),
                         missing=float(rng.uniform(0.0, 0.03)), seed=seed * 1000003 + j + 1))
    return jobs


def serve_cohort(job: dict) -> Cohort:
    """The cohort tables of one serve_stream job."""
    return make_cohort(job["n_ind"], job["n_snp"], n_pop=job["n_pop"], fst=job["fst"], missing=job["missing"],
                       seed=job["seed"])


def window_widths(n_win: int = 4096, lo: int = 500, hi: int = 20000, seed: int = 0) -> np.ndarray:
    """SNP widths of n_win consecutive windows, log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_win))).astype(np.int64)
