"""The allocation-free pass, dpca_pass_fp64_noalloc, against the existing FP64 pass.

This entry point exists for callers that cannot let a library allocate device memory:
applications that hand out all device memory from their own fixed-budget pool, and
latency-sensitive loops in which an allocation, which can synchronise the device, is not
acceptable.  It takes device buffers the caller owns and works in a static device array of the
library.  The test calls it twice in a row through the C ABI, with different start blocks, and
compares each result with a DPCA_PREC_FP64 handle's dpca_pass on the same inputs, within the
FP64 pass tolerance the other tests use (1e-12 relative).  Its device buffers come from torch,
playing the caller that owns the memory.  The file sits last in collection order.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def handle_pass(dpca, packed, n_ind, om):
    with dpca.Handle(n_ind, packed.shape[0], om.shape[1], precision="fp64") as h:
        h.upload(packed)
        h.set_omega(om)
        h.pass_()
        return h.z()


def test_no_alloc_pass_matches_handle_pass_twice(dpca):
    torch = pytest.importorskip("torch")
    from distpca_gb300 import synth

    n_ind, n_snp, k = 1001, 7003, 16  # ragged sizes: n_ind not a multiple of 4, odd SNP count
    c = synth.make_cohort(n_ind, n_snp, n_pop=3, fst=0.05, missing=0.03, seed=11)
    packed = synth.pack_rows(c)  # n_snp x ceil(n_ind / 4) bytes
    np_bytes = packed.shape[1]
    stride = (np_bytes + 31) // 32 * 32
    padded = np.zeros((n_snp, stride), dtype=np.uint8)
    padded[:, :np_bytes] = packed
    dev = torch.device("cuda:0")
    d_packed = torch.from_numpy(padded).to(dev)
    d_z = torch.empty((n_ind, k), dtype=torch.float64, device=dev)
    L = dpca.lib()
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(5)
    for call in range(2):  # two calls in a row share the library's scratch array
        om = rng.standard_normal((n_ind, k))
        d_om = torch.from_numpy(om).to(dev)
        st = L.dpca_pass_fp64_noalloc(ctypes.c_void_p(d_packed.data_ptr()), stride, n_ind, n_snp,
                                      ctypes.c_void_p(d_om.data_ptr()), k, ctypes.c_void_p(d_z.data_ptr()),
                                      ctypes.c_void_p(stream))
        assert st == 0, L.dpca_last_error()
        torch.cuda.synchronize(dev)
        z = d_z.cpu().numpy()
        zr = handle_pass(dpca, packed, n_ind, om)
        assert rel_max(z, zr) < TOL, (call, rel_max(z, zr))


def test_no_alloc_pass_wide_block_and_single_split(dpca):
    """nrhs 128 (the widest block: 64 KB of dynamic shared memory in the X Omega kernel, above the
    default 48 KB limit) on a shape that leaves room for exactly one split of X^T Y partials in
    the 32 MiB array (28,000 SNPs x 128 columns of Y plus per-SNP statistics take ~30.5 MB, one
    split of 2,000 x 128 partials 2 MB), twice in a row."""
    torch = pytest.importorskip("torch")
    from distpca_gb300 import synth

    n_ind, n_snp, k = 2000, 28_000, 128
    fixed = 4 * n_snp * 4 + 2 * n_snp * 8 + 4 * n_snp * 8 + n_snp * k * 8
    part = n_ind * k * 8
    assert fixed + part <= 32 << 20 < fixed + 2 * part  # one split fits, two do not
    c = synth.make_cohort(n_ind, n_snp, n_pop=4, fst=0.05, missing=0.02, seed=23)
    packed = synth.pack_rows(c)
    stride = (packed.shape[1] + 31) // 32 * 32
    padded = np.zeros((n_snp, stride), dtype=np.uint8)
    padded[:, :packed.shape[1]] = packed
    dev = torch.device("cuda:0")
    d_packed = torch.from_numpy(padded).to(dev)
    d_z = torch.empty((n_ind, k), dtype=torch.float64, device=dev)
    L = dpca.lib()
    rng = np.random.default_rng(7)
    for call in range(2):
        om = rng.standard_normal((n_ind, k))
        d_om = torch.from_numpy(om).to(dev)
        st = L.dpca_pass_fp64_noalloc(ctypes.c_void_p(d_packed.data_ptr()), stride, n_ind, n_snp,
                                      ctypes.c_void_p(d_om.data_ptr()), k, ctypes.c_void_p(d_z.data_ptr()), None)
        assert st == 0, L.dpca_last_error()
        torch.cuda.synchronize(dev)
        z = d_z.cpu().numpy()
        zr = handle_pass(dpca, packed, n_ind, om)
        assert rel_max(z, zr) < TOL, (call, rel_max(z, zr))


def test_no_alloc_pass_rejects_sizes_beyond_its_scratch(dpca):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    buf = torch.zeros(1024, dtype=torch.float64, device=dev)
    L = dpca.lib()
    # 200,000 SNPs x nrhs 64 needs ~115 MB of scratch, above the 32 MiB array: rejected before any
    # work is queued (the buffers are never read)
    p = ctypes.c_void_p(buf.data_ptr())
    st = L.dpca_pass_fp64_noalloc(p, 256, 1000, 200_000, p, 64, p, None)
    assert st == 6  # DPCA_ERR_UNSUPPORTED
    assert b"scratch" in L.dpca_last_error()
