"""Host-side logic of libdpca and its C ABI (no GPU compute).

Covers: every symbol declared in include/dpca.h is exported; the start block
is bit-identical to the reference's; flag parsing follows findarg; the
nsv/nrhs/bsize clamps follow distpca.cpp; file probing and its error paths;
the -fwrite writers and the statistics block use the reference's formats.
"""
import ctypes
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, fileset


def declared_symbols():
    with open(os.path.join(ROOT, "include", "dpca.h")) as f:
        text = f.read()
    # function declarations: a return type at the start of a line, then the name and "("
    return sorted(set(re.findall(r"^(?:const\s+)?\w+\s*\*?\s*(dpca_[a-z_0-9]+)\s*\(", text, re.M)))


def test_header_symbols_exported(dpca):
    lib = ctypes.CDLL(dpca.library_path())
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert set(declared_symbols()) == set(dpca.exported_symbols())


@pytest.mark.parametrize("n,k", [(37, 6), (203, 10), (1001, 20), (50000, 2)])
def test_start_block_matches_reference(dpca, golden, n, k):
    om = dpca.start_block(n, k)
    assert hashlib.sha256(om.tobytes()).hexdigest() == str(golden[f"omega_{n}x{k}_sha"])
    if n > 46340:
        np.testing.assert_array_equal(om[42945:42955], golden[f"omega_{n}x{k}_wrap"])


def test_defaults_follow_code_not_readme(dpca):
    c = dpca.config()
    assert (c.nsv, c.nrhs, c.power, c.crit, c.miter, c.verbose, c.fwrite) == (10, 20, 1, 1, 100, 1, 0)
    assert c.tol == 1e-3 and c.prefix == b"noprefix" and c.bsize == 0


def test_findarg_semantics(dpca):
    c, b = dpca.parse_args(["DistPCA.exe", "-bfile", "data/x", "-nsv", "7", "-nsv", "9", "-tol", "1e-6",
                            "-crit", "2", "-prefix", "out", "-power"])
    assert b == "data/x"
    assert c.nsv == 7  # first match wins
    assert c.tol == 1e-6 and c.crit == 2 and c.prefix == b"out"
    assert c.power == 1  # flag without value keeps the default
    c, _ = dpca.parse_args(["x", "-nrhs", "abc"])
    assert c.nrhs == 0  # atoi("abc")
    with pytest.raises(dpca.DpcaError):
        dpca.parse_args(["x", "-precision", "fp8"])


@pytest.mark.parametrize("nsv,nrhs,M,N,exp", [
    (10, 20, 100, 1000, (10, 20)),
    (40, 5, 37, 300, (37, 37)),      # nsv clamps to min(M,N); nrhs < nsv -> min(2 nsv, min)
    (5, 0, 100, 1000, (5, 10)),      # nrhs <= 0 -> min(2 nsv, min(M,N))
    (5, 500, 100, 1000, (5, 100)),   # nrhs > min(M,N) -> min(M,N)
    (8, 6, 100, 1000, (8, 16)),      # nrhs < nsv
])
def test_resolve_clamps(dpca, nsv, nrhs, M, N, exp):
    c = dpca.config(nsv=nsv, nrhs=nrhs, bsize=50)
    rows = dpca.resolve(c, M, N)
    assert (c.nsv, c.nrhs) == exp and rows == 50


def test_resolve_block_size_rules(dpca):
    c = dpca.config(bsize=5000)
    assert dpca.resolve(c, 100, 1000) == 1000  # > local_N -> local_N (in-core)
    c = dpca.config(bsize=0, memory=1e-9)  # no memory to spare -> formula of distpca.cpp:259-260
    rows = dpca.resolve(c, 1000, 100000)
    membuff = 3.0 * 100000 * 8 + 1000 * 10 * 8 + 2.0 * 100000 * 20 + 3.0 * 1000 * 8 + 2048.0 * 100000
    assert rows == int((membuff + 1000 * 8.0) / 1e7)
    c = dpca.config(bsize=0, memory=2.0)
    rows = dpca.resolve(c, 1000, 100000)
    assert rows == 100000  # 2 GB fits the whole matrix -> in-core
    with pytest.raises(dpca.DpcaError):
        dpca.resolve(dpca.config(nsv=0), 10, 10)


def test_probe_counts_and_errors(dpca, tmp_path):
    prefix = os.path.join(GOLDEN, "small")
    assert dpca.probe(prefix) == (203, 2500)
    with pytest.raises(dpca.DpcaError) as e:
        dpca.probe(str(tmp_path / "missing"))
    assert e.value.status == 2
    # bad magic
    p = str(tmp_path / "bad")
    for ext in (".bim", ".fam"):
        with open(prefix + ext) as f, open(p + ext, "w") as g:
            g.write(f.read())
    with open(prefix + ".bed", "rb") as f:
        raw = bytearray(f.read())
    raw[0] = 0x00
    open(p + ".bed", "wb").write(bytes(raw))
    with pytest.raises(dpca.DpcaError) as e:
        dpca.probe(p)
    assert e.value.status == 3
    # individual-major mode byte
    raw[0] = 0x6C
    raw[2] = 0x00
    open(p + ".bed", "wb").write(bytes(raw))
    with pytest.raises(dpca.DpcaError) as e:
        dpca.probe(p)
    assert e.value.status == 3 and "individual-major" in e.value.message
    # truncated .bed
    raw[2] = 0x01
    open(p + ".bed", "wb").write(bytes(raw[:-10]))
    with pytest.raises(dpca.DpcaError) as e:
        dpca.probe(p)
    assert e.value.status == 3
    # .fam whose last line has no newline: not counted (distpca.cpp:137-147)
    open(p + ".bed", "wb").write(bytes(raw))
    with open(prefix + ".fam") as f:
        fam = f.read()
    open(p + ".fam", "w").write(fam + "EXTRA\tX\t0\t0\t0\t-9")
    assert dpca.probe(p) == (203, 2500)


def _fake_result(dpca, n_ind, sigma, u):
    r = dpca.Result()
    r.n_ind, r.nsv = n_ind, len(sigma)
    r.sigma = sigma.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    r.u = u.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    return r


def test_writers_match_reference_format(dpca, golden, tmp_path):
    # feed the reference's own values through our writer: the files must be byte-identical
    prefix = os.path.join(GOLDEN, "small")
    sigma = np.ascontiguousarray(golden["run_small_ooc_sigma"])
    u = np.ascontiguousarray(golden["run_small_ooc_u"])
    c = dpca.config(prefix=str(tmp_path / "r"))
    r = _fake_result(dpca, 203, sigma, u)
    assert dpca.lib().dpca_write_outputs(ctypes.byref(c), prefix.encode(), ctypes.byref(r)) == 0
    for suffix in ("singularValues", "leftSingularVectors"):
        mine = open(str(tmp_path / f"r_{suffix}.txt")).read().splitlines()
        ref = open(os.path.join(GOLDEN, f"small_ooc_ref_{suffix}.txt")).read().splitlines()
        assert mine[: len(ref)] == ref


def test_statistics_block_lines(dpca, tmp_path):
    script = (
        "import ctypes, sys; sys.path.insert(0, %r); import distpca_gb300 as D;"
        "c = D.config(); r = D.Result(); r.n_ind = 942; r.n_snp = 133594; r.nsv = 20; r.nrhs = 40;"
        "r.rows_fetched = 100; r.total_its = 11; r.time_load_matrix = 1.5;"
        "D.lib().dpca_print_statistics(ctypes.byref(c), ctypes.byref(r))" % ROOT)
    out = subprocess.run(["python", "-c", script], capture_output=True, text=True, check=True).stdout
    assert "Total number of times which the data matrix was fetched from the memory: 22" in out
    assert "Total number of matrix rows: 942" in out
    assert "Time to load the data matrix: 1.5000000000000" in out
    assert out.count("Total wall-clock time elapsed:") == 2


def test_no_device_is_a_loud_error(dpca):
    from conftest import gpu_available

    if gpu_available():
        pytest.skip("a GPU is present")
    with pytest.raises(dpca.DpcaError) as e:
        dpca.Handle(100, 100, 4)
    assert e.value.status == 4 and "no CPU fallback" in e.value.message
    prefix, n_ind, n_snp, packed = fileset("tiny")
    with pytest.raises(dpca.DpcaError):
        dpca.decode_counts(packed, n_ind)


def test_full_svd_limits_checked_before_the_device(dpca):
    # the dense check refuses large cohorts up front (no GPU needed to reach the error)
    r = {"sigma": np.ones(3), "u": np.zeros((30_000, 3))}
    packed = np.zeros((4, 7500), dtype=np.uint8)
    with pytest.raises(dpca.DpcaError) as e:
        dpca.full_svd(r, 30_000, 4, packed=packed, nsv=3, nrhs=6)
    assert e.value.status == 6


def test_serving_struct_layouts_match_the_header(dpca, tmp_path):
    """The ctypes mirrors of dpca_serve_config, dpca_job and dpca_job_info have the C layout."""
    import shutil
    import subprocess

    from distpca_gb300 import api

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"dpca_serve_config": api.ServeConfig, "dpca_job": api.Job, "dpca_job_info": api.JobInfo}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "dpca.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.check_call([cc, "-I", os.path.join(root, "include"), str(src), "-o", str(exe)])
    got = dict(line.rsplit(" ", 1) for line in subprocess.check_output([str(exe)]).decode().splitlines())
    for cname, py in structs.items():
        assert int(got[f"{cname} size"]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got[f"{cname} {f}"]) == getattr(py, f).offset, (cname, f)


@pytest.mark.parametrize("k", [1, 2, 3, 8, 20, 40, 97, 128])
def test_sym_eig_matches_numpy(dpca, k):
    """The host Rayleigh-Ritz eigensolver against numpy.linalg.eigh (LAPACK): eigenvalues within
    1e-12 of the largest, eigenvectors orthonormal and A W = W diag(w) to 1e-12 relative."""
    rng = np.random.default_rng(k)
    cases = []
    g = rng.standard_normal((k, k))
    cases.append(g + g.T)                                   # indefinite
    x = rng.standard_normal((3 * k + 5, k))
    cases.append(x.T @ x)                                   # PSD, like Q^T Z
    q, _ = np.linalg.qr(rng.standard_normal((k, k)))
    lam = np.repeat(rng.standard_normal(k // 3 + 1), 3)[:k]
    cases.append((q * lam) @ q.T)                           # clustered / repeated eigenvalues
    cases.append(np.diag(rng.standard_normal(k)))           # already diagonal
    cases.append(np.zeros((k, k)))
    for a in cases:
        upper = np.triu(a) + np.tril(rng.standard_normal((k, k)), -1) * 1e3  # the lower triangle is ignored
        w, W = dpca.sym_eig(upper)
        ref = np.linalg.eigvalsh(a)[::-1]
        scale = max(1.0, np.abs(ref).max())
        assert np.all(np.diff(w) <= 0)
        np.testing.assert_allclose(w, ref, atol=1e-12 * scale, rtol=0)
        np.testing.assert_allclose(W.T @ W, np.eye(k), atol=1e-12)
        assert np.abs(a @ W - W * w).max() <= 1e-12 * scale


@pytest.mark.parametrize("n_ind,n_snp,nrhs,prec,status", [
    (0, 100, 4, "fp64", 1),       # no individuals
    (100, 0, 4, "mixed", 1),      # no SNPs
    (100, 100, 0, "mixed", 1),    # no right-hand sides
    (-5, 100, 4, "fp64", 1),
    (100, 100, 129, "fp64", 6),   # beyond the kernels' nrhs limit
    (100, 100, 4, 7, 1),          # unknown precision
])
def test_empty_and_oversized_shapes_rejected_before_the_device(dpca, n_ind, n_snp, nrhs, prec, status):
    # dpca_create (and its streamed form) validate the shape before any CUDA call, so these
    # status codes are the same with or without a GPU
    for block_snps in (0, 64):
        with pytest.raises(dpca.DpcaError) as e:
            dpca.Handle(n_ind, n_snp, nrhs, precision=prec, block_snps=block_snps)
        assert e.value.status == status, (block_snps, e.value.message)


def test_start_block_rejects_empty_shapes(dpca):
    for n, k in ((0, 4), (10, 0)):
        with pytest.raises(dpca.DpcaError) as e:
            dpca.start_block(n, k)
        assert e.value.status == 1


def test_windows_reject_bad_shapes_before_the_device(dpca):
    # checked before any device work, so these hold without a GPU too
    with pytest.raises(dpca.DpcaError) as e:
        dpca.Windows(500, [1000, 0, 10], 8)
    assert e.value.status == 1
    with pytest.raises(dpca.DpcaError) as e:
        dpca.Windows(500, [1000], 64)
    assert e.value.status == 6


def test_device_utilities_reject_bad_arguments_before_any_device_work(dpca):
    """dpca_qr_device and dpca_sym_eig_device check their arguments first: bad ones return
    DPCA_ERR_INVALID (1) with a message, with or without a GPU."""
    lib = dpca.lib()
    a = np.zeros((4, 2))
    p = a.ctypes.data_as(ctypes.c_void_p)
    assert lib.dpca_qr_device(0, 4, 0, p, 0) == 1  # k = 0
    assert lib.dpca_qr_device(0, 0, 2, p, 0) == 1  # n = 0
    assert lib.dpca_qr_device(0, 4, 2, None, 0) == 1  # no array
    assert lib.dpca_qr_device(0, 4, 100000, p, 0) == 1  # k above the limit
    assert b"dpca_qr_device" in lib.dpca_last_error()
    w = np.zeros(2)
    assert lib.dpca_sym_eig_device(0, 0, p, w.ctypes.data_as(ctypes.c_void_p), p) == 1
    assert lib.dpca_sym_eig_device(0, 2, None, None, None) == 1
