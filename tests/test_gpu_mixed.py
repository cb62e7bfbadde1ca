"""The mixed-precision tcgen05 path against the oracle, the FP64 GPU path and the reference.

Tolerances (written here, derived from the arithmetic): genotypes enter the
tensor cores exactly; Omega and b.Y, a.Y are quantised to 24-bit fixed point per
column (round to nearest, |error| <= 2^-24 of the column maximum) and every
tensor-core sum is an exact integer, folded into FP64.  One pass therefore
agrees with the FP64 result to about 2^-24 times the column max/rms ratio of
the operands (~10 on these cohorts, ~6e-7 of max|Z|); the test allows 3e-6.  Whole solves are held to the targets:
eigenvalues (sigma^2) within 1e-6 relative, largest principal angle of the
nsv-dimensional PC subspace within 1e-4 rad, PC |corr| >= 0.999999 for the
converged leading PCs.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, fileset, run_flags

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def mixed_z(dpca, packed, n_ind, om):
    with dpca.Handle(n_ind, packed.shape[0], om.shape[1], precision="mixed") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        return h.z()


@pytest.mark.parametrize("name,k", [("tiny", 6), ("small", 10), ("wide", 20), ("small", 40)])
def test_pass_matches_oracle(dpca, oracle, name, k):
    prefix, n_ind, n_snp, packed = fileset(name)
    om = dpca.start_block(n_ind, k)
    zr, _ = oracle.one_pass(packed, n_ind, om, bsize=500)
    z = mixed_z(dpca, packed, n_ind, om)
    assert rel_max(z, zr) < 3e-6


@pytest.mark.parametrize("n_ind,n_snp,k", [(5, 7, 2), (129, 513, 3), (517, 2049, 17), (1000, 3001, 40),
                                           (2048, 4099, 48), (3001, 1500, 33), (64, 20000, 8),
                                           (33001, 700, 48), (40000, 1031, 20)])
def test_pass_ragged_shapes_vs_fp64(dpca, n_ind, n_snp, k):
    """Ragged shapes; 33,001 and 40,000 individuals take X Omega's long-K variant (the accumulator
    drained in one copy)."""
    from distpca_gb300 import synth

    c = synth.make_cohort(n_ind, n_snp, n_pop=3, fst=0.05, missing=0.03, seed=n_ind + n_snp)
    packed = synth.pack_rows(c)
    rng = np.random.default_rng(k)
    om = rng.standard_normal((n_ind, k))
    with dpca.Handle(n_ind, n_snp, k, precision="fp64") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        zf = h.z()
    z = mixed_z(dpca, packed, n_ind, om)
    assert rel_max(z, zf) < 3e-6


def test_pass_columns_of_far_apart_magnitudes(dpca):
    """Each Omega column gets its own power-of-two fixed-point scale, and the X Omega epilogue
    removes it by exponent arithmetic: columns from 1e-33 to 1e20 must each match the FP64 pass
    to the per-column tolerance.  At 1e-33 the scale's inverse (~2^-133) is below FP32's normal
    range, so that column takes the epilogue's FP64 branch."""
    from distpca_gb300 import synth

    n_ind, n_snp, k = 700, 3000, 7
    c = synth.make_cohort(n_ind, n_snp, n_pop=3, fst=0.05, missing=0.02, seed=11)
    packed = synth.pack_rows(c)
    om = np.random.default_rng(3).standard_normal((n_ind, k)) * np.array([1e-33, 1e-20, 1e-9, 1.0, 3e5, 1e12, 1e20])
    with dpca.Handle(n_ind, n_snp, k, precision="fp64") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        zf = h.z()
    z = mixed_z(dpca, packed, n_ind, om)
    for j in range(k):
        assert rel_max(z[:, j], zf[:, j]) < 3e-6, j


def test_pass_deterministic(dpca):
    prefix, n_ind, n_snp, packed = fileset("wide")
    om = dpca.start_block(n_ind, 20)
    with dpca.Handle(n_ind, n_snp, 20, precision="mixed") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        a = h.z()
        h.pass_()
        b = h.z()
    assert np.array_equal(a, b)


def subspace_angle(u, v):
    qu, _ = np.linalg.qr(u)
    qv, _ = np.linalg.qr(v)
    s = np.clip(np.linalg.svd(qu.T @ qv, compute_uv=False), -1.0, 1.0)
    return float(np.arccos(s.min()))


@pytest.mark.parametrize("run", ["small_ooc", "small_incore", "small_mev", "wide_mev", "tiny_edges"])
def test_converged_solve_accuracy(dpca, golden, run):
    fl = run_flags(golden, run)
    prefix, n_ind, n_snp, packed = fileset(str(golden[f"run_{run}_fileset"]))
    r = dpca.run(prefix, precision="mixed", nsv=fl["nsv"], nrhs=fl["nrhs"], power=fl.get("power", 1), crit=fl["crit"],
                 tol=fl["tol"], miter=fl.get("miter", 100), bsize=fl["bsize"], verbose=0)
    ref_s, ref_u = golden[f"run_{run}_sigma"], golden[f"run_{run}_u"]
    lam, lam_ref = r["sigma"] ** 2, ref_s ** 2
    assert np.max(np.abs(lam - lam_ref) / lam_ref) < 1e-6
    assert subspace_angle(r["u"], ref_u) < 1e-4
    corr = np.abs(np.sum(r["u"] * ref_u, 0)) / (np.linalg.norm(r["u"], axis=0) * np.linalg.norm(ref_u, axis=0))
    assert corr[:3].min() > 0.999999
    assert abs(r["its"] - int(golden[f"run_{run}_its"])) <= 1


def test_larger_pass_vs_fp64(dpca):
    from distpca_gb300 import synth

    c = synth.make_cohort(20_000, 100_000, n_pop=8, dirichlet=True, fst=0.02, p_range=(0.01, 0.5), missing=0.02,
                          seed=2)
    k = 40
    om = dpca.start_block(c.n_ind, k)
    q, _ = np.linalg.qr(om)
    out = {}
    for prec in ("fp64", "mixed"):
        with dpca.Handle(c.n_ind, c.n_snp, k, precision=prec) as h:
            h.synth_fill(c)
            h.set_omega(q)
            h.pass_()
            out[prec] = h.z()
    err = rel_max(out["mixed"], out["fp64"])
    assert err < 3e-6, err
    # column-wise: the quantisation error is absolute (a fraction of each operand column's
    # maximum), so columns of Z in the bulk of the spectrum, ~40x smaller than the largest
    # ones, see a larger relative error
    col = np.linalg.norm(out["mixed"] - out["fp64"], axis=0) / np.linalg.norm(out["fp64"], axis=0)
    assert col.max() < 2e-5, col


def test_larger_solve_accuracy_vs_fp64(dpca):
    # the solve-level targets at a larger shape: eigenvalues within 1e-6 relative, PC subspace
    # within 1e-4 rad of the FP64 GPU path, same start block and iteration schedule
    from distpca_gb300 import synth

    c = synth.make_cohort(20_000, 100_000, n_pop=8, dirichlet=True, fst=0.02, p_range=(0.01, 0.5), missing=0.02,
                          seed=2)
    packed = synth.pack_rows(c)
    kw = dict(nsv=10, nrhs=20, power=2, crit=1, tol=1e-6, miter=30, bsize=10_000, verbose=0)
    rf = dpca.run_packed(packed, c.n_ind, precision="fp64", **kw)
    rm = dpca.run_packed(packed, c.n_ind, precision="mixed", **kw)
    lam_f, lam_m = rf["sigma"] ** 2, rm["sigma"] ** 2
    assert np.max(np.abs(lam_m - lam_f) / lam_f) < 1e-6
    assert subspace_angle(rm["u"], rf["u"]) < 1e-4


def test_mixed_width_limit(dpca):
    with pytest.raises(dpca.DpcaError) as e:
        dpca.Handle(1000, 1000, 49, precision="mixed")
    assert e.value.status == 6


def test_autotune_keeps_results(dpca):
    """The autotuner changes launch parameters (cluster widths, grid mode, K splits, ring depths)
    and may switch kernels.  With the default kernel kept, the pass result after tuning agrees
    with the default one within 1e-12 (a different K-split count regroups the exact partial sums in
    FP64); after a switch to the G'-product kernel, within that kernel's tolerance (3e-6: X^T Y
    rounds different products to fixed point).  A handle created afterwards for the same shape
    class starts from the tuned choice and agrees with the tuned result within 1e-12."""
    from distpca_gb300 import synth

    n_ind, n_snp, k = 3000, 40_000, 20
    c = synth.make_cohort(n_ind, n_snp, n_pop=4, fst=0.05, missing=0.02, seed=31)
    packed = synth.pack_rows(c)
    om = np.random.default_rng(3).standard_normal((n_ind, k))
    with dpca.Handle(n_ind, n_snp, k, precision="mixed") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        z0 = h.z()
        rep = h.autotune()
        h.set_omega(om)
        h.pass_()
        z1 = h.z()
    for key in ("x_omega_ms", "xt_y_ms", "cluster", "persistent", "kb_per_split", "ring1", "ring2", "x_omega_cluster"):
        assert key in rep
    assert rep["cluster"] in (0, 1, 2, 4) and rep["xt_y_ms"][1] <= rep["xt_y_ms"][0] * 1.05
    assert rep["kernel"] in ("gprod", "products")
    tol = 1e-12 if rep["kernel"] == "products" else 3e-6
    assert np.max(np.abs(z1 - z0)) / np.max(np.abs(z0)) < tol
    with dpca.Handle(n_ind, n_snp, k, precision="mixed") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        assert np.max(np.abs(h.z() - z1)) / np.max(np.abs(z1)) < 1e-12
