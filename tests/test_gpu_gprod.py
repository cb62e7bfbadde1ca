"""The G'-product kernel (genotype product on the tensor cores, missing-genotype term on the CUDA
cores) against the FP64 pass and the two-product kernel.

Both kernels quantise the dense operands to 24-bit fixed point per column and sum exact integers.
X Omega's integers are the same in both (F1 Omega = G' Omega - Miss Omega); X^T Y differs only in
which products are rounded (b.Y and a.Y here, (b-a).Y and a.Y there), so each pass matches the
FP64 pass to the mixed path's tolerance, 3e-6 of max|Z| (test_gpu_mixed.py derives it).  Cases:
  - ordinary cohorts (1-3% missing), ragged shapes, k from 1 to 48, single CTAs and pairs;
  - heavily missing matrices (50%; 90% in a tall-thin shape), where every row's int32 sums are
    folded into the 64-bit sums many times per work item (every 255 missing entries);
  - individuals and SNPs whose genotypes are all missing.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def z_of(dpca, packed, n_ind, om, precision="mixed"):
    with dpca.Handle(n_ind, packed.shape[0], om.shape[1], precision=precision) as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        z1 = h.z()
        h.pass_()
        z2 = h.z()
    assert np.array_equal(z1, z2)  # integer sums: the same bits every pass
    return z1


def three_ways(dpca, monkeypatch, packed, n_ind, om, xw_cl=1, xty_cl=0):
    monkeypatch.setenv("DPCA_XW_CLUSTER", str(xw_cl))
    if xty_cl:
        monkeypatch.setenv("DPCA_XTY_CLUSTER", str(xty_cl))
    zf = z_of(dpca, packed, n_ind, om, "fp64")
    monkeypatch.setenv("DPCA_MIXED_KERNEL", "gprod")
    zg = z_of(dpca, packed, n_ind, om)
    monkeypatch.setenv("DPCA_MIXED_KERNEL", "products")
    zp = z_of(dpca, packed, n_ind, om)
    return zf, zg, zp


@pytest.mark.parametrize("n_ind,n_snp,k,missing,xw_cl,xty_cl", [
    (5, 7, 2, 0.02, 1, 1),
    (517, 3001, 16, 0.02, 1, 1),
    (1000, 4099, 40, 0.03, 2, 2),
    (2048, 20000, 48, 0.01, 1, 2),
    (3001, 1500, 33, 0.01, 2, 1),
    (129, 513, 1, 0.5, 1, 1),
    (3001, 1500, 24, 0.5, 2, 2),
    (64, 20000, 8, 0.9, 1, 1),
])
def test_pass_matches_fp64_and_the_two_product_kernel(dpca, monkeypatch, n_ind, n_snp, k, missing, xw_cl, xty_cl):
    from distpca_gb300 import synth

    c = synth.make_cohort(n_ind, n_snp, n_pop=3, fst=0.05, missing=missing, seed=n_ind * 7 + k)
    packed = synth.pack_rows(c)
    om = np.random.default_rng(k).standard_normal((n_ind, k))
    zf, zg, zp = three_ways(dpca, monkeypatch, packed, n_ind, om, xw_cl, xty_cl)
    assert rel_max(zg, zf) < 3e-6
    assert rel_max(zp, zf) < 3e-6
    assert rel_max(zg, zp) < 3e-6


def test_all_missing_individuals_and_snps(dpca, monkeypatch):
    from distpca_gb300 import synth

    n_ind, n_snp, k = 700, 2500, 12
    c = synth.make_cohort(n_ind, n_snp, n_pop=3, fst=0.05, missing=0.02, seed=5)
    packed = synth.pack_rows(c).copy()
    for i in (0, 3, 131, 699):  # individuals: code 01 in every SNP
        byte, sh = i // 4, 2 * (i % 4)
        packed[:, byte] = (packed[:, byte] & ~np.uint8(3 << sh)) | np.uint8(1 << sh)
    full = n_ind // 4
    for s in (0, 17, 1024, 2499):  # SNPs: code 01 for every individual
        packed[s, :full] = 0x55
        for i in range(4 * full, n_ind):
            sh = 2 * (i % 4)
            packed[s, full] = (packed[s, full] & ~np.uint8(3 << sh)) | np.uint8(1 << sh)
    om = np.random.default_rng(1).standard_normal((n_ind, k))
    zf, zg, zp = three_ways(dpca, monkeypatch, packed, n_ind, om)
    assert np.all(zf[[0, 3, 131, 699]] == 0.0)  # an all-missing individual standardizes to zeros
    assert np.all(zg[[0, 3, 131, 699]] == 0.0)
    assert rel_max(zg, zf) < 3e-6
    assert rel_max(zp, zf) < 3e-6


def test_solve_with_each_kernel(dpca, monkeypatch):
    """A converged solve with either kernel: the same number of iterations and the eigenvalues of
    the FP64 solve within 1e-6 relative."""
    from distpca_gb300 import synth

    n_ind, n_snp = 1500, 30000
    c = synth.make_cohort(n_ind, n_snp, n_pop=4, fst=0.05, missing=0.02, seed=9)
    packed = synth.pack_rows(c)
    flags = dict(nsv=8, nrhs=16, power=2, crit=1, tol=1e-6, miter=60, bsize=n_snp, verbose=0)
    rf = dpca.run_packed(packed, n_ind, precision="fp64", **flags)
    for kern in ("gprod", "products"):
        monkeypatch.setenv("DPCA_MIXED_KERNEL", kern)
        r = dpca.run_packed(packed, n_ind, precision="mixed", **flags)
        assert abs(r["its"] - rf["its"]) <= 1
        lam, lam_f = r["sigma"] ** 2, rf["sigma"] ** 2
        assert np.max(np.abs(lam - lam_f) / lam_f) < 1e-6, kern
