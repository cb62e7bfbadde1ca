"""The CPU oracle (oracle/dpca_oracle.c) against the reference's own outputs.

The golden vectors in tests/golden/golden.npz were produced by the unmodified
reference (oracle/build_ref.sh + tests/golden/make_golden.py).  These tests pin
the C restatement to them before it is trusted as the checker of the GPU path.
"""
import hashlib

import numpy as np
import pytest

from conftest import align_signs, fileset, run_flags


@pytest.mark.parametrize("name", ["tiny", "small", "wide"])
def test_decode_and_standardize_bit_exact(oracle, golden, name):
    prefix, n_ind, n_snp, packed = fileset(name)
    avg, sd, codes = oracle.decode_stats(packed, n_ind, want_codes=True)
    assert np.array_equal(avg.view(np.uint64), golden[f"{name}_avg"].view(np.uint64), equal_nan=False) or \
        np.array_equal(avg, golden[f"{name}_avg"], equal_nan=True)
    np.testing.assert_array_equal(sd, golden[f"{name}_sd"])
    assert hashlib.sha256(codes.tobytes()).hexdigest() == str(golden[f"{name}_dec_sha"])
    np.testing.assert_array_equal(codes[:8], golden[f"{name}_dec_rows"])


def test_standardized_rows_bit_exact(oracle, golden):
    # the standardized values of the first rows and the checksum of all of them
    prefix, n_ind, n_snp, packed = fileset("tiny")
    avg, sd = oracle.decode_stats(packed, n_ind)
    inv = 1.0 / np.sqrt(float(n_snp))
    norm = np.zeros((n_snp, n_ind))
    lut_pre = np.array([3, 1, 2, 0])
    from distpca_gb300 import synth

    codes = synth.unpack_codes(packed, n_ind)
    for s in range(n_snp):
        lut = oracle.lut(avg[s], sd[s])
        norm[s] = lut[lut_pre[codes[s]]] * inv
    np.testing.assert_array_equal(norm[:8], golden["tiny_norm_rows"])
    assert hashlib.sha256(norm.tobytes()).hexdigest() == str(golden["tiny_norm_sha"])


@pytest.mark.parametrize("n,k", [(37, 6), (203, 10), (1001, 20), (50000, 2)])
def test_start_block_bit_exact(oracle, golden, n, k):
    om = oracle.omega(n, k)
    assert hashlib.sha256(om.tobytes()).hexdigest() == str(golden[f"omega_{n}x{k}_sha"])
    np.testing.assert_array_equal(om[:4], golden[f"omega_{n}x{k}_head"])


RUNS = ["small_ooc", "small_incore", "small_mev", "small_trace", "small_fixed3", "tiny_edges", "wide_mev"]


@pytest.mark.parametrize("run", RUNS)
def test_solver_matches_reference(oracle, golden, run):
    fl = run_flags(golden, run)
    prefix, n_ind, n_snp, packed = fileset(str(golden[f"run_{run}_fileset"]))
    r = oracle.solve(packed, n_ind, nsv=fl["nsv"], nrhs=fl["nrhs"], power=fl.get("power", 1), crit=fl["crit"],
                     tol=fl["tol"], miter=fl.get("miter", 100), bsize=fl["bsize"], threads=1)
    ref_sigma = golden[f"run_{run}_sigma"]
    ref_u = golden[f"run_{run}_u"]
    assert r["its"] == int(golden[f"run_{run}_its"])
    # the reference prints 13 decimals; same BLAS calls in the same order
    np.testing.assert_allclose(r["sigma"], ref_sigma, rtol=0, atol=2e-13)
    u = align_signs(r["u"], ref_u)
    np.testing.assert_allclose(u, ref_u, rtol=0, atol=2e-12)


def test_clamped_full_width_run(oracle, golden):
    # -nsv 40 on 37 individuals: nsv and nrhs clamp to 37; the subspace is the whole space,
    # so the singular values are exact and independent of the iteration path
    prefix, n_ind, n_snp, packed = fileset("tiny")
    r = oracle.solve(packed, n_ind, nsv=37, nrhs=37, power=1, crit=1, tol=1e-3, miter=4, bsize=64, threads=1)
    ref = golden["run_tiny_clamp_sigma"]
    assert ref.shape == (37,)
    np.testing.assert_allclose(r["sigma"][:36], ref[:36], rtol=1e-11, atol=2e-13)
