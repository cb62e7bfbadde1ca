"""Out-of-core streaming: the packed rows stay in host memory and are copied in blocks each pass.

A streaming handle (dpca_create_streamed) and a resident one must agree on the same input:
statistics bit-exact; FP64 passes within 1e-12 relative (the block split only regroups the FP64
sums over SNPs); mixed passes within the mixed-pass tolerance 3e-6 of the FP64 pass (each
block's Y operand gets its own 24-bit quantisation scales); whole solves within the solve
targets.  Block sizes are chosen so that the last block is ragged and there are at least three
blocks (both buffers reused).
"""
import numpy as np
import pytest

from conftest import fileset

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def cohort(n_ind, n_snp, seed):
    from distpca_gb300 import synth

    c = synth.make_cohort(n_ind, n_snp, n_pop=4, fst=0.05, missing=0.03, seed=seed)
    return synth.pack_rows(c)


def one_pass(dpca, packed, n_ind, om, precision, block_snps=0):
    with dpca.Handle(n_ind, packed.shape[0], om.shape[1], precision=precision, block_snps=block_snps) as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        return h.z()


def test_streamed_statistics_bit_exact(dpca):
    n_ind, n_snp = 777, 1000
    packed = cohort(n_ind, n_snp, 1)
    out = []
    for blk in (0, 256):
        with dpca.Handle(n_ind, n_snp, 8, precision="fp64", block_snps=blk) as h:
            h.upload(packed)
            out.append(h.snp_stats())
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("n_ind,n_snp,k,blk", [(777, 1000, 8, 256), (1500, 5000, 20, 1280), (300, 4099, 40, 128)])
def test_streamed_fp64_pass_matches_resident(dpca, n_ind, n_snp, k, blk):
    packed = cohort(n_ind, n_snp, n_ind)
    om = np.random.default_rng(k).standard_normal((n_ind, k))
    zr = one_pass(dpca, packed, n_ind, om, "fp64")
    zs = one_pass(dpca, packed, n_ind, om, "fp64", block_snps=blk)
    assert rel_max(zs, zr) < 1e-12


@pytest.mark.parametrize("n_ind,n_snp,k,blk", [(777, 1000, 8, 256), (2000, 9001, 40, 2048), (513, 3000, 17, 384)])
def test_streamed_mixed_pass_matches_fp64(dpca, n_ind, n_snp, k, blk):
    packed = cohort(n_ind, n_snp, n_snp)
    om = np.random.default_rng(k).standard_normal((n_ind, k))
    zr = one_pass(dpca, packed, n_ind, om, "fp64")
    zs = one_pass(dpca, packed, n_ind, om, "mixed", block_snps=blk)
    assert rel_max(zs, zr) < 3e-6


def test_streamed_pass_repeats(dpca):
    # several passes on one streaming handle: the double buffers are reused across passes
    n_ind, n_snp, k = 600, 2000, 12
    packed = cohort(n_ind, n_snp, 3)
    om = np.random.default_rng(9).standard_normal((n_ind, k))
    with dpca.Handle(n_ind, n_snp, k, precision="mixed", block_snps=384) as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        a = h.z()
        h.pass_()
        h.pass_()
        b = h.z()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_streamed_solve_matches_resident(dpca, golden, precision):
    # dpca_run_packed streams when the matrix exceeds the -hbm budget
    prefix, n_ind, n_snp, packed = fileset("small")
    kw = dict(nsv=5, nrhs=10, power=2, crit=1, tol=1e-8, miter=40, bsize=1000, verbose=0, precision=precision)
    rr = dpca.run_packed(packed, n_ind, **kw)
    rs = dpca.run_packed(packed, n_ind, hbm=1e-4, **kw)
    assert rr["streamed"] == 0 and rs["streamed"] == 1
    lam_r, lam_s = rr["sigma"] ** 2, rs["sigma"] ** 2
    if precision == "fp64":
        assert np.max(np.abs(lam_s - lam_r) / lam_r) < 1e-10
        assert rs["its"] == rr["its"]
    else:
        assert np.max(np.abs(lam_s - lam_r) / lam_r) < 1e-6
        qa, _ = np.linalg.qr(rs["u"])
        qb, _ = np.linalg.qr(rr["u"])
        s = np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1.0, 1.0)
        assert float(np.arccos(s.min())) < 1e-4


def test_streamed_handle_rejects_synth_fill(dpca):
    from distpca_gb300 import synth

    c = synth.make_cohort(300, 1000, n_pop=2, fst=0.05, missing=0.01, seed=1)
    with dpca.Handle(300, 1000, 8, precision="fp64", block_snps=256) as h:
        with pytest.raises(dpca.DpcaError) as e:
            h.synth_fill(c)
        assert e.value.status == 6
