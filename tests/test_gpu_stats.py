"""Decode statistics and the device cohort generator on the GPU (bit-exact)."""
import numpy as np
import pytest

from conftest import fileset

pytestmark = pytest.mark.gpu


def code_counts(packed, n_ind):
    from distpca_gb300 import synth

    codes = synth.unpack_codes(packed, n_ind)
    return np.stack([(codes == c).sum(1) for c in range(4)], axis=1).astype(np.int32)


@pytest.mark.parametrize("name", ["tiny", "small", "wide"])
def test_counts_mean_sd_bit_exact(dpca, oracle, golden, name):
    prefix, n_ind, n_snp, packed = fileset(name)
    counts, avg, sd = dpca.decode_counts(packed, n_ind)
    np.testing.assert_array_equal(counts, code_counts(packed, n_ind))
    ref_avg, ref_sd = golden[f"{name}_avg"], golden[f"{name}_sd"]
    # bit-exact, NaN where every genotype is missing
    assert np.array_equal(avg, ref_avg, equal_nan=True)
    assert np.array_equal(sd, ref_sd, equal_nan=True)
    o_avg, o_sd = oracle.decode_stats(packed, n_ind)
    assert np.array_equal(avg, o_avg, equal_nan=True) and np.array_equal(sd, o_sd, equal_nan=True)


def test_lut_bit_exact(dpca, oracle):
    prefix, n_ind, n_snp, packed = fileset("tiny")
    with dpca.Handle(n_ind, n_snp, 4, precision="fp64") as h:
        h.upload(packed)
        counts, avg, sd, lut = h.snp_stats()
    inv = 1.0 / np.sqrt(float(n_snp))
    for s in range(n_snp):
        ref = oracle.lut(avg[s], sd[s])  # indexed by {3,1,2,0}[code]
        expect = np.array([ref[3], ref[1], ref[2], ref[0]]) * inv
        assert np.array_equal(lut[s], expect), s


@pytest.mark.parametrize("n_ind", [1, 2, 3, 5, 63, 64, 65, 127, 129, 515])
def test_ragged_individual_counts(dpca, oracle, n_ind):
    from distpca_gb300 import synth

    c = synth.make_cohort(n_ind, 67, n_pop=1, missing=0.1, seed=n_ind)
    packed = synth.pack_rows(c)
    packed[:, -1] |= 0xFF ^ ((1 << (2 * (n_ind % 4 or 4))) - 1) & 0xFF  # garbage in the pad bits
    counts, avg, sd = dpca.decode_counts(packed, n_ind)
    np.testing.assert_array_equal(counts, code_counts(packed, n_ind))
    o_avg, o_sd = oracle.decode_stats(packed, n_ind)
    assert np.array_equal(avg, o_avg, equal_nan=True) and np.array_equal(sd, o_sd, equal_nan=True)


@pytest.mark.parametrize("n_ind,n_snp", [(37, 11), (1000, 300), (4099, 129)])
def test_device_generator_matches_numpy(dpca, n_ind, n_snp):
    from distpca_gb300 import synth

    c = synth.make_cohort(n_ind, n_snp, n_pop=3, dirichlet=True, missing=0.03, heavy_frac=0.1, heavy_rate=0.5,
                          seed=n_ind)
    with dpca.Handle(n_ind, n_snp, 2, precision="fp64") as h:
        h.synth_fill(c)
        dev = h.download_packed()
        counts, _, _, _ = h.snp_stats()
    ref = synth.pack_rows(c)
    np.testing.assert_array_equal(dev, ref)
    np.testing.assert_array_equal(counts, code_counts(ref, n_ind))


def test_stats_at_scale_sum_of_counts(dpca):
    # size-independent property at a large shape: counts add up to n_ind per SNP
    from distpca_gb300 import synth

    c = synth.make_cohort(50_001, 2_000, n_pop=8, dirichlet=True, fst=0.02, p_range=(0.01, 0.5), missing=0.02,
                          seed=2)
    with dpca.Handle(c.n_ind, c.n_snp, 2, precision="fp64") as h:
        h.synth_fill(c)
        counts, avg, sd, lut = h.snp_stats()
        rows = h.download_packed(1990, 2000)
    assert (counts.sum(1) == c.n_ind).all()
    np.testing.assert_array_equal(counts[1990:], code_counts(rows, c.n_ind))
    assert abs(counts[:, 1].sum() / counts.sum() - 0.02) < 0.001
