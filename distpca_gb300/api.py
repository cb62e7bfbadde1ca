"""ctypes mirror of the libdpca C ABI (include/dpca.h).

The names follow the reference's solver interface: ``run`` is the drop-in for
``BlockSubspaceIter_MPI_OOC_double_buffering`` / ``SubspaceIteration_MPI``
(driven by the same flags as DistPCA.exe), ``Handle`` keeps a genotype matrix
resident on the GPU, ``start_block`` reproduces the reference's Gaussian start
block bit for bit.  Nothing here computes on the CPU: every numeric call goes
to the CUDA library, and loading fails loudly when it has not been built.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Optional, Sequence

import numpy as np

__all__ = ["DpcaError", "Config", "Result", "Handle", "lib", "library_path", "config", "parse_args", "probe",
           "resolve", "start_block", "run", "run_packed", "decode_counts", "PREC_FP64", "PREC_MIXED",
           "exported_symbols", "FullSVD", "full_svd", "Server", "JobInfo", "sym_eig", "qr_device", "Windows"]

HERE = os.path.dirname(os.path.abspath(__file__))
PREC_FP64 = 0
PREC_MIXED = 1

_STATUS = {0: "ok", 1: "invalid argument", 2: "I/O error", 3: "bad input format", 4: "CUDA error",
           5: "out of memory", 6: "unsupported shape", 7: "device wait timed out", 8: "numerical failure"}


class DpcaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS.get(status, status)}: {message}")
        self.status = status
        self.message = message


class Config(ctypes.Structure):
    _fields_ = [("nsv", ctypes.c_int), ("nrhs", ctypes.c_int), ("power", ctypes.c_int), ("crit", ctypes.c_int),
                ("miter", ctypes.c_int), ("bsize", ctypes.c_int), ("verbose", ctypes.c_int),
                ("fwrite", ctypes.c_int), ("full_svd", ctypes.c_int), ("tol", ctypes.c_double),
                ("memory_gb", ctypes.c_double), ("prefix", ctypes.c_char * 1024), ("precision", ctypes.c_int),
                ("device", ctypes.c_int), ("hbm_budget_gb", ctypes.c_double)]


_D = ctypes.POINTER(ctypes.c_double)
# dpca_block_fn: int fn(void *ctx, int64_t first_snp, int n_rows, const uint8_t **rows, int64_t *row_stride)
BLOCK_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                            ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64))


class Result(ctypes.Structure):
    _fields_ = [("n_ind", ctypes.c_int), ("n_snp", ctypes.c_int), ("nsv", ctypes.c_int), ("nrhs", ctypes.c_int),
                ("rows_fetched", ctypes.c_int), ("total_its", ctypes.c_int), ("passes", ctypes.c_int),
                ("in_core", ctypes.c_int), ("streamed", ctypes.c_int), ("sigma", _D), ("u", _D),
                ("delta_iter", _D), ("time_generate_rhs", ctypes.c_double), ("time_load_matrix", ctypes.c_double),
                ("time_mm", ctypes.c_double), ("time_mm_a", ctypes.c_double), ("time_mm_a_t", ctypes.c_double),
                ("time_gs", ctypes.c_double), ("time_projected_svd", ctypes.c_double),
                ("time_other", ctypes.c_double), ("time_total", ctypes.c_double),
                ("time_true_svd", ctypes.c_double), ("frob_norm_angle", ctypes.c_double),
                ("cos_error", ctypes.c_double)]


def library_path() -> str:
    return os.environ.get("DPCA_LIBRARY", os.path.join(HERE, "_build", "libdpca.so"))


class ServeConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("slots", ctypes.c_int), ("hbm_budget_gb", ctypes.c_double)]


class Job(ctypes.Structure):
    _fields_ = [("n_ind", ctypes.c_int), ("n_snp", ctypes.c_int), ("cfg", Config), ("packed", ctypes.c_void_p),
                ("row_stride", ctypes.c_int64), ("synth_key", ctypes.c_uint64), ("synth_pop", ctypes.c_void_p),
                ("synth_miss_thr", ctypes.c_void_p), ("synth_snp_thr", ctypes.c_void_p), ("synth_n_pop", ctypes.c_int),
                ("omega", ctypes.c_void_p), ("sigma", ctypes.c_void_p), ("u", ctypes.c_void_p)]


class JobInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("total_its", ctypes.c_int), ("passes", ctypes.c_int),
                ("t_submit", ctypes.c_double), ("t_start", ctypes.c_double), ("t_done", ctypes.c_double),
                ("device_gb", ctypes.c_double), ("error", ctypes.c_char * 256)]


_lib = None

_SIGS = {
    "dpca_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "dpca_last_error": (ctypes.c_char_p, []),
    "dpca_version": (ctypes.c_char_p, []),
    "dpca_config_init": (None, [ctypes.POINTER(Config)]),
    "dpca_parse_args": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(Config),
                                       ctypes.c_char_p, ctypes.c_size_t]),
    "dpca_probe_bfile": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "dpca_resolve_config": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int)]),
    "dpca_start_block": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "dpca_sym_eig": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "dpca_sym_eig_device": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "dpca_qr_device": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    "dpca_run": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_char_p, ctypes.c_void_p, ctypes.POINTER(Result)]),
    "dpca_run_packed": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(Result)]),
    "dpca_write_outputs": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_char_p, ctypes.POINTER(Result)]),
    "dpca_print_statistics": (None, [ctypes.POINTER(Config), ctypes.POINTER(Result)]),
    "dpca_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "dpca_create_streamed": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    "dpca_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dpca_upload": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "dpca_upload_file": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "dpca_inject_fault": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]),
    "dpca_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "dpca_upload_blocks": (ctypes.c_int, [ctypes.c_void_p, BLOCK_FN, ctypes.c_void_p, ctypes.c_int64]),
    "dpca_synth_fill": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int]),
    "dpca_download_packed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "dpca_snp_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]),
    "dpca_set_omega": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dpca_pass": (ctypes.c_int, [ctypes.c_void_p]),
    "dpca_get_z": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dpca_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Config), ctypes.c_void_p, ctypes.POINTER(Result)]),
    "dpca_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "dpca_kernel_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
    "dpca_reset_kernel_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dpca_pass_fp64_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "dpca_full_svd": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "dpca_write_fullsvd": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p]),
    "dpca_decode_counts": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "dpca_windows_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "dpca_windows_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dpca_windows_upload": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "dpca_windows_synth_fill": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_int]),
    "dpca_windows_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Config), ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]),
    "dpca_windows_handle": (ctypes.c_void_p, [ctypes.c_void_p]),
    "dpca_serve_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ServeConfig)]),
    "dpca_serve_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_int64)]),
    "dpca_serve_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(JobInfo)]),
    "dpca_serve_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.POINTER(JobInfo)]),
    "dpca_serve_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "dpca_serve_shutdown": (ctypes.c_int, [ctypes.c_void_p]),
}


def exported_symbols() -> Sequence[str]:
    return list(_SIGS)


def lib():
    """Load libdpca.so (raises if it has not been built: there is no fallback)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise ImportError(f"libdpca.so not found at {path}; build it with "
                              "`python -c 'import __graft_entry__ as g; g.build()'` or distpca_gb300/build.py")
        L = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(st: int) -> None:
    if st != 0:
        raise DpcaError(st, lib().dpca_last_error().decode(errors="replace"))


def _p(a: Optional[np.ndarray]):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


_ALIASES = {"memory": "memory_gb", "fullSVD": "full_svd", "hbm": "hbm_budget_gb"}


def config(**kw) -> Config:
    """Defaults of DistPCA.exe (initialize_structure) overridden by keyword flags."""
    c = Config()
    lib().dpca_config_init(ctypes.byref(c))
    fields = {name for name, _ in Config._fields_}
    for k, v in kw.items():
        k = _ALIASES.get(k, k)
        if k not in fields:
            raise TypeError(f"unknown flag {k!r}")
        if k == "prefix":
            c.prefix = v.encode()
        elif k == "precision" and isinstance(v, str):
            c.precision = {"fp64": PREC_FP64, "mixed": PREC_MIXED}[v]
        else:
            setattr(c, k, v)
    return c


def parse_args(argv: Sequence[str]):
    c = config()
    arr = (ctypes.c_char_p * len(argv))(*[a.encode() for a in argv])
    buf = ctypes.create_string_buffer(1024)
    _check(lib().dpca_parse_args(len(argv), arr, ctypes.byref(c), buf, 1024))
    return c, buf.value.decode()


def probe(bfile: str):
    m, n = ctypes.c_int(0), ctypes.c_int(0)
    _check(lib().dpca_probe_bfile(bfile.encode(), ctypes.byref(m), ctypes.byref(n)))
    return m.value, n.value


def resolve(c: Config, n_ind: int, n_snp: int) -> int:
    rows = ctypes.c_int(0)
    _check(lib().dpca_resolve_config(ctypes.byref(c), n_ind, n_snp, ctypes.byref(rows)))
    return rows.value


def start_block(n_ind: int, k: int) -> np.ndarray:
    out = np.empty((n_ind, k), dtype=np.float64)
    _check(lib().dpca_start_block(n_ind, k, _p(out)))
    return out


def sym_eig(b: np.ndarray, device: Optional[int] = None):
    """Eigenvalues (descending) and eigenvectors (columns) of the symmetric matrix b (upper triangle
    used): the Rayleigh-Ritz eigenproblem, on the host (dsyev's method), or with the device kernel
    the solve uses when `device` is given."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    k = b.shape[0]
    w = np.empty(k)
    W = np.empty((k, k))
    if device is None:
        _check(lib().dpca_sym_eig(k, _p(b), _p(w), _p(W)))
    else:
        _check(lib().dpca_sym_eig_device(device, k, _p(b), _p(w), _p(W)))
    return w, W


def qr_device(a: np.ndarray, device: int = 0, separate: bool = False) -> np.ndarray:
    """Q of the thin QR of the n x k panel a with the device kernels every solve uses (shifted
    CholeskyQR3); `separate` runs it as separate kernels instead of one cooperative launch."""
    q = np.array(a, dtype=np.float64, order="C", copy=True)
    n, k = q.shape
    _check(lib().dpca_qr_device(device, n, k, _p(q), 1 if separate else 0))
    return q


def _result_arrays(c: Config, n_ind: int):
    sigma = np.zeros(c.nsv)
    u = np.zeros((n_ind, c.nsv))
    delta = np.zeros(max(c.miter, 1))
    r = Result()
    r.sigma = sigma.ctypes.data_as(_D)
    r.u = u.ctypes.data_as(_D)
    r.delta_iter = delta.ctypes.data_as(_D)
    return r, sigma, u, delta


def _result_dict(r: Result, sigma, u, delta, omega) -> Dict:
    d = {name: getattr(r, name) for name, _ in Result._fields_ if name not in ("sigma", "u", "delta_iter")}
    d.update(sigma=sigma, u=u, delta_iter=delta[: r.total_its], omega=omega, its=r.total_its)
    return d


def run(bfile: str, omega0: Optional[np.ndarray] = None, **flags) -> Dict:
    """Full solve of <bfile>.bed/.bim/.fam with DistPCA.exe flags as keywords."""
    c = config(**flags)
    n_ind, n_snp = probe(bfile)
    resolve(c, n_ind, n_snp)
    omega = start_block(n_ind, c.nrhs) if omega0 is None else np.array(omega0, dtype=np.float64, order="C")
    r, sigma, u, delta = _result_arrays(c, n_ind)
    _check(lib().dpca_run(ctypes.byref(c), bfile.encode(), _p(omega), ctypes.byref(r)))
    if c.fwrite == 1:
        _check(lib().dpca_write_outputs(ctypes.byref(c), bfile.encode(), ctypes.byref(r)))
    return _result_dict(r, sigma, u, delta, omega)


def run_packed(packed: np.ndarray, n_ind: int, omega0: Optional[np.ndarray] = None, **flags) -> Dict:
    """Full solve from packed SNP-major rows held in host memory."""
    packed = np.ascontiguousarray(packed, dtype=np.uint8)
    c = config(**flags)
    n_snp = packed.shape[0]
    resolve(c, n_ind, n_snp)
    omega = start_block(n_ind, c.nrhs) if omega0 is None else np.array(omega0, dtype=np.float64, order="C")
    r, sigma, u, delta = _result_arrays(c, n_ind)
    _check(lib().dpca_run_packed(ctypes.byref(c), _p(packed), packed.shape[1], n_ind, n_snp, _p(omega),
                                 ctypes.byref(r)))
    return _result_dict(r, sigma, u, delta, omega)


def decode_counts(packed: np.ndarray, n_ind: int):
    """Per-SNP code counts {00, 01, 10, 11}, avg and sd computed on the GPU."""
    packed = np.ascontiguousarray(packed, dtype=np.uint8)
    n_snp = packed.shape[0]
    counts = np.zeros((n_snp, 4), dtype=np.int32)
    avg = np.zeros(n_snp)
    sd = np.zeros(n_snp)
    _check(lib().dpca_decode_counts(_p(packed), packed.shape[1], n_ind, n_snp, _p(counts), _p(avg), _p(sd)))
    return counts, avg, sd


class Handle:
    """A genotype matrix on one GPU plus the subspace state.

    block_snps > 0 makes a streaming handle: the rows stay in host memory (the array given to
    upload, kept referenced here) and every pass copies them in blocks of block_snps SNPs.
    """

    def __init__(self, n_ind: int, n_snp: int, nrhs: int, precision=PREC_MIXED, device: int = 0,
                 stream: Optional[int] = None, block_snps: int = 0):
        if isinstance(precision, str):
            precision = {"fp64": PREC_FP64, "mixed": PREC_MIXED}[precision]
        self.n_ind, self.n_snp, self.nrhs, self.precision = n_ind, n_snp, nrhs, precision
        self._host = None
        h = ctypes.c_void_p()
        st = ctypes.c_void_p(stream) if stream else None
        if block_snps > 0:
            _check(lib().dpca_create_streamed(ctypes.byref(h), n_ind, n_snp, nrhs, precision, device, st, block_snps))
        else:
            _check(lib().dpca_create(ctypes.byref(h), n_ind, n_snp, nrhs, precision, device, st))
        self._h = h

    def close(self) -> None:
        if self._h:
            lib().dpca_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, packed: np.ndarray) -> None:
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        assert packed.shape[0] == self.n_snp
        self._host = packed  # a streaming handle reads these rows in every pass
        _check(lib().dpca_upload(self._h, _p(packed), packed.shape[1]))

    def upload_ptr(self, ptr: int, row_stride: int) -> None:
        _check(lib().dpca_upload(self._h, ctypes.c_void_p(ptr), row_stride))

    def autotune(self) -> Dict:
        """Tune the product kernels' launch parameters on this handle (see dpca_autotune)."""
        import json

        buf = ctypes.create_string_buffer(1024)
        _check(lib().dpca_autotune(self._h, buf, 1024))
        return json.loads(buf.value.decode())

    def inject_fault(self, fault: int = 1, wait_limit_ms: float = 1.0) -> None:
        """Test hook: the next mixed X Omega launch withholds one load; its bounded wait runs out."""
        _check(lib().dpca_inject_fault(self._h, fault, wait_limit_ms))

    def upload_file(self, bed_path: str) -> None:
        """Rows from a SNP-major .bed through the library's block reader (read every pass when
        streaming)."""
        _check(lib().dpca_upload_file(self._h, bed_path.encode()))

    def upload_blocks(self, fn, max_row_stride: int) -> None:
        """Rows handed out by fn(first_snp, n_rows) -> (host address, row stride) per block."""

        def cb(ctx, s0, rows, out_ptr, out_stride):
            try:
                ptr, stride = fn(int(s0), int(rows))
            except Exception:
                return 1
            out_ptr[0] = ptr
            out_stride[0] = stride
            return 0

        self._blocks_cb = BLOCK_FN(cb)  # kept alive for as long as the handle may call it
        _check(lib().dpca_upload_blocks(self._h, self._blocks_cb, None, max_row_stride))

    def synth_fill(self, cohort) -> None:
        pop = np.ascontiguousarray(cohort.pop, dtype=np.uint8)
        miss = np.ascontiguousarray(cohort.miss_thr, dtype=np.uint32)
        thr = np.ascontiguousarray(cohort.snp_thr, dtype=np.uint32)
        _check(lib().dpca_synth_fill(self._h, ctypes.c_uint64(cohort.key), _p(pop), _p(miss), _p(thr),
                                     cohort.n_pop))

    def download_packed(self, s0: int = 0, s1: Optional[int] = None) -> np.ndarray:
        s1 = self.n_snp if s1 is None else s1
        out = np.empty((s1 - s0, (self.n_ind + 3) // 4), dtype=np.uint8)
        _check(lib().dpca_download_packed(self._h, s0, s1, _p(out)))
        return out

    def snp_stats(self):
        counts = np.zeros((self.n_snp, 4), dtype=np.int32)
        avg = np.zeros(self.n_snp)
        sd = np.zeros(self.n_snp)
        lut = np.zeros((self.n_snp, 4))
        _check(lib().dpca_snp_stats(self._h, _p(counts), _p(avg), _p(sd), _p(lut)))
        return counts, avg, sd, lut

    def set_omega(self, omega: np.ndarray) -> None:
        om = np.ascontiguousarray(omega, dtype=np.float64)
        assert om.shape == (self.n_ind, self.nrhs)
        _check(lib().dpca_set_omega(self._h, _p(om)))

    def pass_(self) -> None:
        _check(lib().dpca_pass(self._h))

    def z(self) -> np.ndarray:
        out = np.empty((self.n_ind, self.nrhs))
        _check(lib().dpca_get_z(self._h, _p(out)))
        return out

    def synchronize(self) -> None:
        _check(lib().dpca_synchronize(self._h))

    def solve(self, omega0: Optional[np.ndarray] = None, **flags) -> Dict:
        c = config(nrhs=self.nrhs, precision=self.precision, **flags)
        if c.bsize <= 0:
            c.bsize = self.n_snp
        omega = start_block(self.n_ind, self.nrhs) if omega0 is None else np.array(omega0, dtype=np.float64,
                                                                                      order="C")
        r, sigma, u, delta = _result_arrays(c, self.n_ind)
        r.rows_fetched = c.bsize
        _check(lib().dpca_solve(self._h, ctypes.byref(c), _p(omega), ctypes.byref(r)))
        return _result_dict(r, sigma, u, delta, omega)

    def kernel_times(self) -> Dict[str, Dict[str, float]]:
        cap = 64
        names = ctypes.create_string_buffer(8192)
        ms = np.zeros(cap)
        launches = np.zeros(cap, dtype=np.int64)
        count = ctypes.c_int(0)
        _check(lib().dpca_kernel_times(self._h, names, 8192, _p(ms), _p(launches), ctypes.byref(count), cap))
        keys = names.value.decode().split(";") if count.value else []
        return {k: {"ms": float(ms[i]), "launches": int(launches[i])} for i, k in enumerate(keys)}

    def reset_kernel_times(self, enable: bool = True) -> None:
        _check(lib().dpca_reset_kernel_times(self._h, 1 if enable else 0))


class FullSVD(ctypes.Structure):
    _fields_ = [("info", ctypes.c_int), ("time_true_svd", ctypes.c_double), ("frob_norm_angle", ctypes.c_double),
                ("cos_error", ctypes.c_double), ("true_sigma", _D), ("true_u", _D), ("sigma_relerr", _D),
                ("vec_relerr", _D), ("cosines", _D)]


def full_svd(result: Dict, n_ind: int, n_snp: int, packed: Optional[np.ndarray] = None, bfile: Optional[str] = None,
             write: bool = False, **flags) -> Dict:
    """-fullSVD check of a result (sigma, u) against the dense SVD of the standardized matrix."""
    c = config(**flags)
    nsv = len(result["sigma"])
    sigma = np.ascontiguousarray(result["sigma"], dtype=np.float64)
    u = np.ascontiguousarray(result["u"], dtype=np.float64)
    r = Result()
    r.n_ind, r.n_snp, r.nsv, r.nrhs = n_ind, n_snp, nsv, c.nrhs
    r.sigma = sigma.ctypes.data_as(_D)
    r.u = u.ctypes.data_as(_D)
    out = {k: np.zeros(n) for k, n in (("true_sigma", nsv), ("true_u", n_ind * nsv), ("sigma_relerr", nsv),
                                         ("vec_relerr", n_ind * nsv), ("cosines", nsv))}
    f = FullSVD()
    for k, a in out.items():
        setattr(f, k, a.ctypes.data_as(_D))
    if packed is not None:
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        st = lib().dpca_full_svd(ctypes.byref(c), None, _p(packed), packed.shape[1], n_ind, n_snp, ctypes.byref(r),
                                 ctypes.byref(f))
    else:
        st = lib().dpca_full_svd(ctypes.byref(c), bfile.encode(), None, 0, n_ind, n_snp, ctypes.byref(r),
                                 ctypes.byref(f))
    _check(st)
    if write:
        _check(lib().dpca_write_fullsvd(ctypes.byref(c), bfile.encode() if bfile else None, n_ind, nsv,
                                        ctypes.byref(f)))
    out["true_u"] = out["true_u"].reshape(n_ind, nsv)
    out["vec_relerr"] = out["vec_relerr"].reshape(n_ind, nsv)
    out.update(info=f.info, time_true_svd=f.time_true_svd, frob_norm_angle=f.frob_norm_angle, cos_error=f.cos_error)
    return out


class Server:
    """The serving loop (dpca_serve_*): independent PCA jobs, up to `slots` in flight on one GPU.

    submit() takes packed host rows or a synthetic cohort (distpca_gb300.synth.Cohort) and the
    run flags; it returns a job id at once.  The arrays a job reads and writes are kept referenced
    here until the job has been waited for.  result(job) waits and returns the job's
    {"sigma", "u", "its", "passes", "info"}.
    """

    def __init__(self, device: int = 0, slots: int = 4, hbm_gb: float = 0.0):
        c = ServeConfig(device, slots, hbm_gb)
        s = ctypes.c_void_p()
        _check(lib().dpca_serve_create(ctypes.byref(s), ctypes.byref(c)))
        self._s = s
        self._keep: Dict[int, tuple] = {}

    def submit(self, n_ind: int, n_snp: int, packed: Optional[np.ndarray] = None, cohort=None,
               omega0: Optional[np.ndarray] = None, want_u: bool = True, **flags) -> int:
        c = config(**flags)
        j = Job()
        j.n_ind, j.n_snp, j.cfg = n_ind, n_snp, c
        keep = []
        if packed is not None:
            packed = np.ascontiguousarray(packed, dtype=np.uint8)
            assert packed.shape[0] == n_snp
            j.packed, j.row_stride = packed.ctypes.data, packed.shape[1]
            keep.append(packed)
        else:
            pop = np.ascontiguousarray(cohort.pop, dtype=np.uint8)
            miss = np.ascontiguousarray(cohort.miss_thr, dtype=np.uint32)
            thr = np.ascontiguousarray(cohort.snp_thr, dtype=np.uint32)
            j.synth_key, j.synth_n_pop = cohort.key, cohort.n_pop
            j.synth_pop, j.synth_miss_thr, j.synth_snp_thr = pop.ctypes.data, miss.ctypes.data, thr.ctypes.data
            keep += [pop, miss, thr]
        if omega0 is not None:
            omega0 = np.ascontiguousarray(omega0, dtype=np.float64)
            assert omega0.shape == (n_ind, c.nrhs)
            j.omega = omega0.ctypes.data
            keep.append(omega0)
        sigma = np.zeros(c.nsv)
        u = np.zeros((n_ind, c.nsv)) if want_u else None
        j.sigma = sigma.ctypes.data
        j.u = u.ctypes.data if u is not None else None
        jid = ctypes.c_int64(0)
        _check(lib().dpca_serve_submit(self._s, ctypes.byref(j), ctypes.byref(jid)))
        self._keep[jid.value] = (keep, sigma, u)
        return jid.value

    def poll(self, job: int) -> bool:
        done = ctypes.c_int(0)
        _check(lib().dpca_serve_poll(self._s, job, ctypes.byref(done), None))
        return bool(done.value)

    def wait(self, job: int, timeout: float = -1.0) -> JobInfo:
        info = JobInfo()
        _check(lib().dpca_serve_wait(self._s, job, timeout, ctypes.byref(info)))
        return info

    def result(self, job: int, timeout: float = -1.0) -> Dict:
        info = self.wait(job, timeout)
        keep, sigma, u = self._keep.pop(job)
        if info.status != 0:
            raise DpcaError(info.status, info.error.decode(errors="replace"))
        return {"sigma": sigma, "u": u, "its": info.total_its, "passes": info.passes, "info": info}

    def stats(self) -> Dict:
        done, mif, peak, budget = ctypes.c_int64(0), ctypes.c_int(0), ctypes.c_double(0), ctypes.c_double(0)
        _check(lib().dpca_serve_stats(self._s, ctypes.byref(done), ctypes.byref(mif), ctypes.byref(peak),
                                      ctypes.byref(budget)))
        return {"done": done.value, "max_in_flight": mif.value, "peak_gb": peak.value, "budget_gb": budget.value}

    def shutdown(self) -> None:
        if self._s:
            lib().dpca_serve_shutdown(self._s)
            self._s = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.shutdown()

    def __del__(self):
        try:
            self.shutdown()
        except Exception:
            pass


class Windows:
    """Batched local PCA (dpca_windows_*): independent PCAs of consecutive SNP windows that share
    the individuals, solved together on one GPU.  win_snps[w] SNPs per window, in row order."""

    def __init__(self, n_ind: int, win_snps: Sequence[int], nrhs: int, device: int = 0, stream: Optional[int] = None):
        self.n_ind, self.nrhs = n_ind, nrhs
        self.win_snps = np.ascontiguousarray(win_snps, dtype=np.int32)
        self.n_win = len(self.win_snps)
        w = ctypes.c_void_p()
        st = ctypes.c_void_p(stream) if stream else None
        _check(lib().dpca_windows_create(ctypes.byref(w), n_ind, self.n_win, _p(self.win_snps), nrhs, device, st))
        self._w = w

    @property
    def n_snp(self) -> int:
        return int(self.win_snps.sum())

    def close(self) -> None:
        if getattr(self, "_w", None):
            lib().dpca_windows_destroy(self._w)
            self._w = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, packed: np.ndarray) -> None:
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        assert packed.shape[0] == self.n_snp
        _check(lib().dpca_windows_upload(self._w, _p(packed), packed.shape[1]))

    def synth_fill(self, cohort) -> None:
        assert cohort.n_snp == self.n_snp and cohort.n_ind == self.n_ind
        pop = np.ascontiguousarray(cohort.pop, dtype=np.uint8)
        miss = np.ascontiguousarray(cohort.miss_thr, dtype=np.uint32)
        thr = np.ascontiguousarray(cohort.snp_thr, dtype=np.uint32)
        _check(lib().dpca_windows_synth_fill(self._w, ctypes.c_uint64(cohort.key), _p(pop), _p(miss), _p(thr),
                                             cohort.n_pop))

    def solve(self, omega0: Optional[np.ndarray] = None, want_u: bool = True, **flags) -> Dict:
        c = config(nrhs=self.nrhs, **flags)
        om = None if omega0 is None else np.ascontiguousarray(omega0, dtype=np.float64)
        sigma = np.zeros((self.n_win, c.nsv))
        u = np.zeros((self.n_win, self.n_ind, c.nsv)) if want_u else None
        its = np.zeros(self.n_win, dtype=np.int32)
        _check(lib().dpca_windows_solve(self._w, ctypes.byref(c), _p(om), _p(sigma), _p(u), _p(its)))
        return {"sigma": sigma, "u": u, "its": its}

    def handle(self) -> int:
        return lib().dpca_windows_handle(self._w)

    def kernel_times(self) -> Dict[str, Dict[str, float]]:
        cap = 64
        names = ctypes.create_string_buffer(8192)
        ms = np.zeros(cap)
        launches = np.zeros(cap, dtype=np.int64)
        count = ctypes.c_int(0)
        _check(lib().dpca_kernel_times(ctypes.c_void_p(self.handle()), names, 8192, _p(ms), _p(launches),
                                       ctypes.byref(count), cap))
        keys = names.value.decode().split(";") if count.value else []
        return {k: {"ms": float(ms[i]), "launches": int(launches[i])} for i, k in enumerate(keys)}

    def reset_kernel_times(self, enable: bool = True) -> None:
        _check(lib().dpca_reset_kernel_times(ctypes.c_void_p(self.handle()), 1 if enable else 0))
