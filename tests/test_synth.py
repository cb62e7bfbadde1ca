"""The seeded Balding-Nichols generator (host side)."""
import numpy as np

from distpca_gb300 import synth


def test_pack_unpack_round_trip():
    rng = np.random.default_rng(0)
    for n in (1, 3, 4, 37, 128, 1001):
        codes = rng.integers(0, 4, size=(5, n), dtype=np.uint8)
        packed = synth.pack_codes(codes)
        assert packed.shape == (5, (n + 3) // 4)
        np.testing.assert_array_equal(synth.unpack_codes(packed, n), codes)


def test_deterministic_and_blockwise():
    c = synth.make_cohort(301, 500, n_pop=3, fst=0.05, missing=0.02, seed=7)
    a = synth.pack_rows(c)
    b = synth.pack_rows(synth.make_cohort(301, 500, n_pop=3, fst=0.05, missing=0.02, seed=7))
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a[123:200], synth.pack_rows(c, 123, 200))
    assert not np.array_equal(a, synth.pack_rows(synth.make_cohort(301, 500, n_pop=3, seed=8)))


def test_model_statistics():
    c = synth.make_cohort(4000, 300, n_pop=4, fst=0.02, p_range=(0.1, 0.5), missing=0.03, seed=3)
    codes = synth.genotype_codes(c, 0, 300)
    miss = codes == 1
    assert abs(miss.mean() - 0.03) < 0.003
    g = np.array([0, 0, 1, 2])[codes]
    freq = (g * ~miss).sum(1) / (2 * (~miss).sum(1))
    pk = c.snp_thr.astype(np.float64) / 2**32
    expect = (pk[:, c.pop]).mean(1)
    assert np.abs(freq - expect).max() < 0.05
    # heterozygotes follow HWE within each population
    het = (codes == 2).sum(1) / (~miss).sum(1)
    assert np.abs(het - (2 * pk * (1 - pk))[:, c.pop].mean(1)).max() < 0.05


def test_heavy_missing_layout():
    c = synth.make_cohort(2000, 50, n_pop=2, missing=0.0, heavy_frac=0.1, heavy_rate=0.5, seed=1)
    codes = synth.genotype_codes(c, 0, 50)
    per_ind = (codes == 1).mean(0)
    assert (per_ind > 0.2).sum() == 200
    assert abs((codes == 1).mean() - 0.05) < 0.01


def test_write_and_read_plink(tmp_path):
    c = synth.make_cohort(10, 7, n_pop=2, seed=2)
    packed = synth.pack_rows(c)
    prefix = str(tmp_path / "x")
    synth.write_plink(prefix, packed, 10)
    raw = open(prefix + ".bed", "rb").read()
    assert raw[:3] == bytes([0x6C, 0x1B, 0x01]) and len(raw) == 3 + 7 * 3
    np.testing.assert_array_equal(synth.read_bed(prefix, 10, 7), packed)
    assert len(open(prefix + ".fam").read().splitlines()) == 10


def test_c_generator_matches_numpy():
    from oracle import oracle as O

    c = synth.make_cohort(203, 300, n_pop=4, dirichlet=True, missing=0.05, heavy_frac=0.1, heavy_rate=0.4, seed=4)
    np.testing.assert_array_equal(O.synth_rows(c, 17, 300), synth.pack_rows(c, 17, 300))
