"""Failure detection on the device, without faulting the GPU.

Every barrier wait in the tcgen05 product kernel is bounded.  dpca_inject_fault makes one launch's
load producer withhold a batch, so that the MMA issuer's wait for it runs out (after 1 ms here
instead of the normal ~4 s); the kernel records the site, waits for its own copies and MMAs in
flight, frees its tensor memory and returns.  What must hold afterwards: the call that reads the
result reports DPCA_ERR_TIMEOUT, the same handle's next pass is correct (the CUDA context is
intact), and so is a fresh handle's.  The reference has no failure detection (errors abort the MPI
job, read statuses are unchecked: methods.cpp:803, 811).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def case(oracle):
    from distpca_gb300 import synth

    n_ind, n_snp, k = 517, 3001, 16
    c = synth.make_cohort(n_ind, n_snp, n_pop=4, fst=0.05, missing=0.02, seed=1)
    packed = synth.pack_rows(c)
    import distpca_gb300 as D

    om = D.start_block(n_ind, k)
    zr, _ = oracle.one_pass(packed, n_ind, om, bsize=1000)
    return n_ind, n_snp, k, packed, om, zr


def test_withheld_load_times_out_and_the_handle_recovers(dpca, case):
    n_ind, n_snp, k, packed, om, zr = case
    with dpca.Handle(n_ind, n_snp, k, precision="mixed") as h:
        h.upload(packed)
        h.set_omega(om)
        h.inject_fault(1, wait_limit_ms=1.0)
        h.pass_()
        with pytest.raises(dpca.DpcaError) as e:
            h.z()
        assert e.value.status == 7 and "gave up" in str(e.value)
        h.pass_()  # the fault applied to one launch only
        assert rel_max(h.z(), zr) < 1e-5
    with dpca.Handle(n_ind, n_snp, k, precision="mixed") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        assert rel_max(h.z(), zr) < 1e-5


def test_solve_reports_the_timeout(dpca, case):
    n_ind, n_snp, k, packed, om, zr = case
    with dpca.Handle(n_ind, n_snp, k, precision="mixed") as h:
        h.upload(packed)
        h.inject_fault(1, wait_limit_ms=1.0)
        with pytest.raises(dpca.DpcaError) as e:
            h.solve(om, nsv=4, power=2, crit=1, tol=1e-6, miter=5, bsize=1000)
        assert e.value.status == 7
        r = h.solve(om, nsv=4, power=2, crit=1, tol=1e-6, miter=5, bsize=1000)
        assert np.isfinite(r["sigma"]).all() and r["sigma"][0] > 0


def test_fault_hook_arguments_are_checked(dpca, case):
    n_ind, n_snp, k, packed, om, zr = case
    with dpca.Handle(n_ind, n_snp, k, precision="fp64") as h:
        with pytest.raises(dpca.DpcaError) as e:
            h.inject_fault(1, 1.0)
        assert e.value.status == 6
    with dpca.Handle(n_ind, n_snp, k, precision="mixed") as h:
        for bad in ((2, 1.0), (1, 0.0), (1, -3.0)):
            with pytest.raises(dpca.DpcaError):
                h.inject_fault(*bad)
