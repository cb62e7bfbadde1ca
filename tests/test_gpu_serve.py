"""The serving loop (dpca_serve_*): many independent PCA jobs of uneven size on one GPU.

What the loop promises, each checked here:
  - a job's result is the same alone and in the mix: submitted alone to a server, or together
    with jobs of other sizes, nsv and precisions that overlap it on the device, its singular
    values and vectors are bit-identical (the kernels are deterministic and jobs share no device
    state), and they agree with a plain dpca_solve of the same inputs within the tolerances the
    solve tests use (1e-10 relative for FP64 sigma, 1e-6 for mixed; PC |corr| >= 0.999999);
  - jobs overlap: with several slots, jobs submitted together are in flight at the same time;
  - admission respects the memory budget, and a job larger than the whole budget fails with
    DPCA_ERR_NOMEM without running;
  - jobs with packed host rows work as well as synthetic ones;
  - bad job descriptions are rejected at submission.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLAGS = dict(power=2, crit=2, tol=1e-3, miter=6)


def cohorts():
    from distpca_gb300 import synth

    # (n_ind, n_snp, nsv, precision): uneven sizes, nsv and precisions
    specs = [(1500, 20000, 5, "mixed"), (700, 9000, 3, "fp64"), (2600, 31000, 8, "mixed"),
             (1100, 14000, 4, "mixed"), (520, 12000, 5, "fp64"), (3300, 24000, 6, "mixed")]
    out = []
    for i, (n, m, nsv, prec) in enumerate(specs):
        c = synth.make_cohort(n, m, n_pop=2 + i % 4, fst=0.03 + 0.01 * i, missing=0.01 * (i % 3), seed=100 + i)
        out.append((c, dict(nsv=nsv, nrhs=2 * nsv, precision=prec, bsize=m, **FLAGS)))
    return out


def submit_all(server, jobs):
    return [server.submit(c.n_ind, c.n_snp, cohort=c, **f) for c, f in jobs]


def test_results_same_alone_and_in_the_mix(dpca):
    jobs = cohorts()
    alone = []
    with dpca.Server(slots=4) as s:  # same server settings for both runs
        for c, f in jobs:
            alone.append(s.result(s.submit(c.n_ind, c.n_snp, cohort=c, **f)))
        ids = submit_all(s, jobs)
        mixed = [s.result(j) for j in ids]
        st = s.stats()
    assert st["max_in_flight"] >= 2
    for a, b in zip(alone, mixed):
        assert np.array_equal(a["sigma"], b["sigma"])
        assert np.array_equal(a["u"], b["u"])
        assert a["its"] == b["its"]


def test_results_match_plain_solve(dpca):
    jobs = cohorts()[:4]
    with dpca.Server(slots=3) as s:
        ids = submit_all(s, jobs)
        got = [s.result(j) for j in ids]
    for (c, f), r in zip(jobs, got):
        run_flags = {k: v for k, v in f.items() if k not in ("nrhs", "precision")}
        with dpca.Handle(c.n_ind, c.n_snp, f["nrhs"], precision=f["precision"]) as h:
            h.synth_fill(c)
            ref = h.solve(dpca.start_block(c.n_ind, f["nrhs"]), **run_flags)
        lam, lam_r = r["sigma"] ** 2, ref["sigma"] ** 2
        tol = 1e-10 if f["precision"] == "fp64" else 1e-6
        assert np.max(np.abs(lam - lam_r) / lam_r) < tol
        corr = np.abs(np.sum(r["u"] * ref["u"], axis=0)) / (
            np.linalg.norm(r["u"], axis=0) * np.linalg.norm(ref["u"], axis=0))
        assert corr.min() >= 0.999999


def test_jobs_overlap_on_the_device(dpca):
    jobs = cohorts()
    with dpca.Server(slots=4) as s:
        ids = submit_all(s, jobs)
        infos = [s.result(j)["info"] for j in ids]
    spans = sorted((i.t_start, i.t_done) for i in infos)
    overlapping = sum(1 for a, b in zip(spans, spans[1:]) if b[0] < a[1])
    assert overlapping >= 1
    assert all(i.t_submit <= i.t_start <= i.t_done for i in infos)


def test_admission_respects_the_budget(dpca):
    jobs = cohorts()
    need = []
    with dpca.Server(slots=4) as s:
        for c, f in jobs[:2]:
            need.append(s.result(s.submit(c.n_ind, c.n_snp, cohort=c, **f))["info"].device_gb)
    budget = 1.2 * max(need)  # room for about one job at a time
    with dpca.Server(slots=4, hbm_gb=budget) as s:
        ids = submit_all(s, jobs[:2] * 2)
        for j in ids:
            s.result(j)
        st = s.stats()
        assert st["peak_gb"] <= budget + 1e-9
        assert abs(st["budget_gb"] - budget) < 1e-6
        # a job larger than the whole budget fails at submission time, without running
        from distpca_gb300 import synth

        big = synth.make_cohort(20000, 200000, n_pop=2, fst=0.05, missing=0.0, seed=9)
        jid = s.submit(big.n_ind, big.n_snp, cohort=big, nsv=5, nrhs=10, precision="mixed", **FLAGS)
        with pytest.raises(dpca.DpcaError) as e:
            s.result(jid)
        assert e.value.status == 5


def test_packed_host_job_matches_synthetic(dpca):
    from distpca_gb300 import synth

    c, f = cohorts()[1]
    packed = synth.pack_rows(c)
    with dpca.Server(slots=2) as s:
        a = s.result(s.submit(c.n_ind, c.n_snp, cohort=c, **f))
        b = s.result(s.submit(c.n_ind, c.n_snp, packed=packed, **f))
    assert np.array_equal(a["sigma"], b["sigma"])
    assert np.array_equal(a["u"], b["u"])


def test_bad_jobs_rejected_at_submission(dpca):
    c, f = cohorts()[0]
    with dpca.Server(slots=1) as s:
        with pytest.raises(dpca.DpcaError) as e:
            s.submit(c.n_ind, c.n_snp, cohort=c, **{**f, "nsv": 30})  # nsv > nrhs
        assert e.value.status == 1
        with pytest.raises(dpca.DpcaError):
            s.submit(c.n_ind, c.n_snp, packed=np.zeros((c.n_snp, 2), np.uint8), **f)  # rows too short


def test_jobs_match_oracle(dpca, oracle):
    """Three jobs of the mixed stream (one FP64, two mixed) against the CPU oracle (the reference's
    algorithm restated in C, pinned to the reference build) solving the same rows with the same
    flags and start block: eigenvalues within 1e-10 (FP64) / 1e-6 (mixed) relative, the largest
    principal angle between the nsv-dimensional subspaces within 1e-6 / 1e-4 rad, iteration
    counts equal (FP64) or within one (mixed).  The jobs stop at MEV tol 1e-3 after at most six
    iterations, so their trailing directions still carry the rounding noise of the reference's
    nearly rank-deficient start block (3.7e-8 rad measured for the FP64 job)."""
    from distpca_gb300 import synth

    jobs = [cohorts()[i] for i in (0, 1, 3)]
    packs = [synth.pack_rows(c) for c, _ in jobs]
    with dpca.Server(slots=3) as s:
        ids = [s.submit(c.n_ind, c.n_snp, packed=p, **f) for (c, f), p in zip(jobs, packs)]
        got = [s.result(j) for j in ids]
    for (c, f), p, r in zip(jobs, packs, got):
        ref = oracle.solve(p, c.n_ind, nsv=f["nsv"], nrhs=f["nrhs"], power=f["power"], crit=f["crit"], tol=f["tol"],
                           miter=f["miter"], bsize=f["bsize"])
        fp64 = f["precision"] == "fp64"
        lam, lam_r = r["sigma"] ** 2, ref["sigma"] ** 2
        assert np.max(np.abs(lam - lam_r) / lam_r) < (1e-10 if fp64 else 1e-6)
        qa, _ = np.linalg.qr(r["u"])
        qb, _ = np.linalg.qr(ref["u"])
        ang = float(np.arccos(np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False).min(), -1, 1)))
        assert ang < (1e-6 if fp64 else 1e-4), ang
        assert abs(r["its"] - ref["its"]) <= (0 if fp64 else 1), (r["its"], ref["its"])
