"""The plain FP64 GPU path against the oracle and the reference's own results.

Tolerances: the FP64 path uses the reference's standardized values bit for bit
and FP64 products in a different summation order than OpenBLAS, so one pass
agrees to ~1e-13 relative.  Whole solves agree on the iteration count; the
three leading singular values (well separated, converged) to 1e-10 relative
and their PC vectors to |corr| >= 1 - 1e-10.  Trailing, unconverged
components are as sensitive to rounding as the reference itself: its own
singular values move by up to 3.8e-8 relative between BLAS thread counts on
these fixtures (small_fixed3), so they are held to 5e-8 and |corr| >= 1 - 1e-5.
The reference's start block is nearly rank-deficient (kappa ~ 5e9: entry (j, c) reseeds
the LCG with j*n_ind + c, so neighbouring columns are almost parallel); after only
three iterations every singular value still carries that rounding noise (the
reference varies by 4.7e-8 with its own thread count), so short fixed-iteration runs
are held to 2e-7.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, align_signs, fileset, run_flags

pytestmark = pytest.mark.gpu

RUNS = ["small_ooc", "small_incore", "small_mev", "small_trace", "small_fixed3", "tiny_edges", "wide_mev"]


def rel_max(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name,k", [("tiny", 6), ("small", 10), ("wide", 20)])
def test_one_pass_matches_oracle(dpca, oracle, name, k):
    prefix, n_ind, n_snp, packed = fileset(name)
    om = dpca.start_block(n_ind, k)
    zr, _ = oracle.one_pass(packed, n_ind, om, bsize=97)
    with dpca.Handle(n_ind, n_snp, k, precision="fp64") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        z = h.z()
    assert rel_max(z, zr) < 1e-12


def test_pass_is_deterministic(dpca):
    prefix, n_ind, n_snp, packed = fileset("small")
    om = dpca.start_block(n_ind, 12)
    with dpca.Handle(n_ind, n_snp, 12, precision="fp64") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        a = h.z()
        h.pass_()
        b = h.z()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("run", RUNS)
def test_solve_matches_reference(dpca, golden, run):
    fl = run_flags(golden, run)
    prefix, n_ind, n_snp, packed = fileset(str(golden[f"run_{run}_fileset"]))
    r = dpca.run(prefix, precision="fp64", nsv=fl["nsv"], nrhs=fl["nrhs"], power=fl.get("power", 1), crit=fl["crit"],
                 tol=fl["tol"], miter=fl.get("miter", 100), bsize=fl["bsize"], verbose=0)
    assert r["its"] == int(golden[f"run_{run}_its"])
    assert r["in_core"] == (1 if fl["bsize"] >= n_snp else 0)
    tol_lead, tol_all = (2e-7, 2e-7) if run == "small_fixed3" else (1e-10, 5e-8)
    check_against(r, golden[f"run_{run}_sigma"], golden[f"run_{run}_u"], tol_lead=tol_lead, tol_all=tol_all)


def check_against(r, ref_s, ref_u, lead=3, tol_lead=1e-10, tol_all=5e-8):
    rel = np.abs(r["sigma"] - ref_s) / ref_s
    assert rel[:lead].max() < tol_lead, rel
    assert rel.max() < tol_all, rel
    u = align_signs(r["u"], ref_u)
    corr = np.abs(np.sum(u * ref_u, 0)) / (np.linalg.norm(u, axis=0) * np.linalg.norm(ref_u, axis=0))
    assert corr[:lead].min() > 1 - max(1e-10, tol_lead), corr
    assert corr.min() > 1 - 1e-5, corr


def test_full_width_clamped_run(dpca, golden):
    prefix = os.path.join(GOLDEN, "tiny")
    r = dpca.run(prefix, precision="fp64", nsv=40, nrhs=5, bsize=64, crit=1, tol=1e-3, miter=4, verbose=0)
    assert r["sigma"].shape == (37,)
    # the subspace is the whole space: these are the exact singular values
    np.testing.assert_allclose(r["sigma"][:36], golden["run_tiny_clamp_sigma"][:36], rtol=1e-10)


def test_run_packed_equals_run(dpca):
    prefix, n_ind, n_snp, packed = fileset("small")
    kw = dict(precision="fp64", nsv=5, nrhs=10, crit=1, tol=-1, miter=3, bsize=700, verbose=0)
    a = dpca.run(prefix, **kw)
    b = dpca.run_packed(packed, n_ind, **kw)
    assert np.array_equal(a["sigma"], b["sigma"]) and np.array_equal(a["u"], b["u"])


def test_cli_drop_in(dpca, golden, tmp_path):
    from distpca_gb300 import build as B

    exe = B.CLI
    out = subprocess.run([exe, "-bfile", os.path.join(GOLDEN, "small"), "-nsv", "5", "-nrhs", "10", "-power", "2",
                          "-crit", "1", "-tol", "1e-6", "-bsize", "400", "-fwrite", "1", "-verbose", "2",
                          "-prefix", str(tmp_path / "r"), "-precision", "fp64"], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "Total number of times which the data matrix was fetched from the memory: %d" % (
        3 * int(golden["run_small_ooc_its"])) in out.stdout
    crit_lines = [ln for ln in out.stdout.splitlines() if ln.startswith("Iteration ")]
    assert crit_lines == list(golden["run_small_ooc_crit"])
    sv = np.loadtxt(str(tmp_path / "r_singularValues.txt"))
    np.testing.assert_allclose(sv, golden["run_small_ooc_sigma"], rtol=5e-8)
    lines = open(str(tmp_path / "r_leftSingularVectors.txt")).read().splitlines()
    ref = open(os.path.join(GOLDEN, "small_ooc_ref_leftSingularVectors.txt")).read().splitlines()
    assert lines[0] == ref[0] and len(lines) == 204
    assert [ln.split("\t")[0] for ln in lines[1:11]] == [ln.split("\t")[0] for ln in ref[1:11]]


def test_cli_errors_exit_nonzero(dpca, tmp_path):
    from distpca_gb300 import build as B

    out = subprocess.run([B.CLI, "-bfile", str(tmp_path / "nope")], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "Error reading file" in out.stdout


def test_unsupported_width_is_reported(dpca):
    with pytest.raises(dpca.DpcaError) as e:
        dpca.Handle(1000, 1000, 129)
    assert e.value.status == 6


@pytest.mark.parametrize("k", [64, 96, 128])
def test_wide_subspace_pass(dpca, oracle, k):
    # widths whose shared-memory tiles pass the default 48 KB limit
    prefix, n_ind, n_snp, packed = fileset("wide")
    om = np.random.default_rng(k).standard_normal((n_ind, k))
    zr, _ = oracle.one_pass(packed, n_ind, om, bsize=300)
    with dpca.Handle(n_ind, n_snp, k, precision="fp64") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        z = h.z()
    assert rel_max(z, zr) < 1e-12
