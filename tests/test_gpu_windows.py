"""Batched local PCA over SNP windows (dpca_windows_*).

Each window is an independent PCA of its SNP rows (standardized with 1/sqrt(window width)),
solved together with the others.  A window's result must be the one a resident handle of its
rows alone gives with the same flags (dpca_solve, mixed precision, bsize < n_snp): eigenvalues
within 1e-6 relative (the mixed-path tolerance), PCs |corr| >= 0.999999, the same number of outer
iterations (the per-window convergence test stops each window on its own).  Windows of uneven
widths that are not multiples of the 512-row padding exercise the padded layout; host rows and
the on-device synthesis must give identical results.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WIDTHS = [600, 1300, 517, 2048, 900, 3001, 512, 777]
FLAGS = dict(nsv=2, power=3, crit=1, tol=1e-5, miter=12)


def cohort(n_ind, widths, seed=7):
    from distpca_gb300 import synth

    return synth.make_cohort(n_ind, int(sum(widths)), n_pop=4, fst=0.05, missing=0.01, seed=seed)


def alone(dpca, packed, n_ind, s0, s1, nrhs, flags):
    with dpca.Handle(n_ind, s1 - s0, nrhs, precision="mixed") as h:
        h.upload(packed[s0:s1])
        return h.solve(dpca.start_block(n_ind, nrhs), bsize=s1 - s0 - 1, **flags)


def corr_min(a, b):
    return float((np.abs(np.sum(a * b, 0)) / (np.linalg.norm(a, axis=0) * np.linalg.norm(b, axis=0))).min())


@pytest.mark.parametrize("n_ind,nrhs", [(700, 8), (1029, 12)])
def test_windows_match_single_solves(dpca, n_ind, nrhs):
    from distpca_gb300 import synth

    c = cohort(n_ind, WIDTHS)
    packed = synth.pack_rows(c)
    with dpca.Windows(n_ind, WIDTHS, nrhs) as w:
        w.synth_fill(c)
        r = w.solve(**FLAGS)
    offs = np.concatenate([[0], np.cumsum(WIDTHS)])
    for i in range(len(WIDTHS)):
        ref = alone(dpca, packed, n_ind, offs[i], offs[i + 1], nrhs, FLAGS)
        lam, lam_r = r["sigma"][i] ** 2, ref["sigma"] ** 2
        assert np.max(np.abs(lam - lam_r) / lam_r) < 1e-6, i
        assert corr_min(r["u"][i], ref["u"]) >= 0.999999, i
        assert r["its"][i] == ref["its"], (i, r["its"][i], ref["its"])


def test_windows_upload_equals_synth(dpca):
    from distpca_gb300 import synth

    n_ind = 900
    c = cohort(n_ind, WIDTHS, seed=3)
    packed = synth.pack_rows(c)
    out = []
    for mode in ("synth", "upload"):
        with dpca.Windows(n_ind, WIDTHS, 8) as w:
            w.synth_fill(c) if mode == "synth" else w.upload(packed)
            out.append(w.solve(**FLAGS))
    assert np.array_equal(out[0]["sigma"], out[1]["sigma"])
    assert np.array_equal(out[0]["u"], out[1]["u"])
    assert np.array_equal(out[0]["its"], out[1]["its"])


@pytest.mark.parametrize("crit,tol", [(0, 1e-4), (2, 1e-3)])
def test_windows_other_criteria(dpca, crit, tol):
    from distpca_gb300 import synth

    n_ind = 640
    widths = WIDTHS[:5]
    c = cohort(n_ind, widths, seed=11)
    packed = synth.pack_rows(c)
    flags = dict(nsv=2, power=2, crit=crit, tol=tol, miter=10)
    with dpca.Windows(n_ind, widths, 8) as w:
        w.synth_fill(c)
        r = w.solve(**flags)
    offs = np.concatenate([[0], np.cumsum(widths)])
    for i in range(len(widths)):
        ref = alone(dpca, packed, n_ind, offs[i], offs[i + 1], 8, flags)
        assert np.max(np.abs(r["sigma"][i] ** 2 - ref["sigma"] ** 2) / ref["sigma"] ** 2) < 1e-6
        assert r["its"][i] == ref["its"]



def max_angle(u, ref):
    qa, _ = np.linalg.qr(u)
    qb, _ = np.linalg.qr(ref)
    s = np.linalg.svd(qa.T @ qb, compute_uv=False)
    return float(np.arccos(np.clip(s.min(), -1.0, 1.0)))


def test_windows_match_oracle(dpca, oracle):
    """Three windows of uneven width against the CPU oracle (the reference's algorithm restated in
    C, pinned to the reference build) solving each window's rows alone: a window is its own PCA,
    standardized with 1/sqrt(width), so the oracle's solve of those rows is the reference result
    for it.  Mixed-path gates: eigenvalues within 1e-6 relative, the largest principal angle
    between the nsv-dimensional subspaces within 1e-4 rad, iteration counts within one."""
    from distpca_gb300 import synth

    n_ind, nrhs = 806, 8
    widths = [1300, 3001, 777]
    c = synth.make_cohort(n_ind, int(sum(widths)), n_pop=3, fst=0.08, missing=0.01, seed=21)
    packed = synth.pack_rows(c)
    flags = dict(nsv=2, power=3, crit=1, tol=1e-6, miter=20)
    with dpca.Windows(n_ind, widths, nrhs) as w:
        w.upload(packed)
        r = w.solve(**flags)
    offs = np.concatenate([[0], np.cumsum(widths)])
    for i in range(len(widths)):
        s0, s1 = int(offs[i]), int(offs[i + 1])
        ref = oracle.solve(packed[s0:s1], n_ind, nrhs=nrhs, bsize=s1 - s0 - 1, **flags)
        lam, lam_r = r["sigma"][i] ** 2, ref["sigma"] ** 2
        assert np.max(np.abs(lam - lam_r) / lam_r) < 1e-6, (i, lam, lam_r)
        assert max_angle(r["u"][i], ref["u"]) < 1e-4, i
        assert abs(int(r["its"][i]) - ref["its"]) <= 1, (i, r["its"][i], ref["its"])
