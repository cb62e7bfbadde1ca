"""-fullSVD: the dense SVD check (distpca.cpp:449-635) against the reference's own run.

The reference computes LAPACKE_dgesvd of the n_ind x n_snp standardized matrix; the device
check takes the eigendecomposition of the FP64 Gram matrix X^T X.  Leading singular values agree
within 1e-10 relative (the Gram form's error on a singular value is ~eps * sigma_max^2 / sigma,
far below that for the leading ones), |left singular vectors| within 1e-8, and |cosines| between
the same approximate and true vectors within 1e-6.  Fixture: tests/golden/make_golden_fullsvd.py.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, fileset

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    return np.load(os.path.join(GOLDEN, "small_fullsvd.npz"))


def flags_of(ref):
    f = list(ref["flags"])
    return {"nsv": int(f[1]), "nrhs": int(f[3]), "power": int(f[5]), "crit": int(f[7]), "tol": float(f[9]),
            "bsize": int(f[11])}


def test_full_svd_matches_reference(dpca, ref):
    prefix, n_ind, n_snp, packed = fileset("small")
    kw = flags_of(ref)
    r = dpca.run_packed(packed, n_ind, precision="fp64", verbose=0, **kw)
    out = dpca.full_svd(r, n_ind, n_snp, packed=packed, **kw)
    assert out["info"] == 0
    ts = ref["true_sigma"]
    assert np.max(np.abs(out["true_sigma"] - ts) / ts) < 1e-10
    assert np.max(np.abs(np.abs(out["true_u"]) - ref["true_u_abs"])) < 1e-8
    assert np.max(np.abs(np.abs(out["cosines"]) - np.abs(ref["cosines"]))) < 1e-6
    # the same approximate vectors: errors consistent with the cosines
    np.testing.assert_allclose(out["sigma_relerr"], np.abs(out["true_sigma"] - r["sigma"]) / out["true_sigma"])
    assert out["frob_norm_angle"] >= 0 and out["cos_error"] >= 0


def test_cli_full_svd_files(dpca, ref, tmp_path):
    exe = os.path.join(os.path.dirname(dpca.library_path()), "dpca")
    kw = [str(x) for x in ref["flags"]]
    pref = str(tmp_path / "out")
    cmd = [exe, "-bfile", os.path.join(GOLDEN, "small"), "-fwrite", "1", "-fullSVD", "1", "-verbose", "2",
           "-precision", "fp64", "-prefix", pref] + kw
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "FULL SVD computed in" in r.stdout and "RelError Sigma(4):" in r.stdout and "Cosine(4):" in r.stdout
    n_ind = 203
    for name, lines in (("realSingularValues", 5), ("realLeftSingularVectors", n_ind), ("singvecs_accuracy", n_ind * 5),
                        ("cosineValues", 5)):
        with open(f"{pref}_{name}.txt") as f:
            got = f.read().splitlines()
        with open(os.path.join(GOLDEN, f"small_fullsvd_ref_{name}.txt")) as f:
            want = f.read().splitlines()
        assert len(got) == lines
        # same layout: fields per line, fixed 13-digit formats, trailing separator of the vectors file
        for g, w in zip(got[:3], want[:3]):
            assert len(g.split(" ")) == len(w.split(" "))
            assert all(len(x.split(".")[-1]) == 13 for x in g.split())
    true_sigma = np.loadtxt(f"{pref}_realSingularValues.txt")
    assert np.max(np.abs(true_sigma - ref["true_sigma"]) / ref["true_sigma"]) < 1e-10
