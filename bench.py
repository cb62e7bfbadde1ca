#!/usr/bin/env python
"""Genotypes/s per power iteration (one pass Z = X^T X Omega) on GB300.

Workload (default): the in-core mixed-precision configuration -- 50,000
individuals x 1,000,000 SNPs (12.5 GB packed, HBM-resident), seeded
Balding-Nichols cohort (K=8 populations, Dirichlet(1) sizes, Fst 0.02,
p ~ U(0.01, 0.5), 2% missing), nrhs 40.  A step is one pass over the whole
matrix; the packed matrix (12.5 GB) is far larger than L2, so no flush is
needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl dpca|reference]

N > 1 runs N independent replicas (one per GPU; the path has no data-path
collective) and reports the whole-job throughput.  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "genotypes/s per power iter, mixed vs FP64 GPU @PC err≤1e-6; serve p50/p99"
UNIT = "genotypes/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["dpca", "reference"], default="dpca")
    p.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    p.add_argument("--n-ind", type=int, default=50_000)
    p.add_argument("--n-snp", type=int, default=1_000_000)
    p.add_argument("--nrhs", type=int, default=40)
    p.add_argument("--power", type=int, default=6)
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--cpu-snps", type=int, default=20_000, help="SNP rows in the CPU baseline sample")
    p.add_argument("--fp64-snps", type=int, default=50_000, help="SNP rows for the plain FP64 GPU comparison")
    p.add_argument("--accuracy-snps", type=int, default=100_000, help="SNP rows for the mixed-vs-FP64 accuracy solve")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-extras", action="store_true", help="skip the FP64 comparison and the accuracy solve")
    p.add_argument("--no-serve", action="store_true", help="skip the serving-loop job stream")
    p.add_argument("--no-windows", action="store_true", help="skip the batched-window local PCA")
    p.add_argument("--windows", type=int, default=4096, help="SNP windows in the batched local PCA")
    p.add_argument("--serve-jobs", type=int, default=512)
    p.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate (jobs/s)")
    p.add_argument("--serve-slots", type=int, default=8)
    p.add_argument("--serve-sample", type=int, default=8, help="jobs in the one-at-a-time FP64 comparison")
    return p.parse_args()


# ----------------------------------------------------------------------------- ranks
class Ranks:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.dist = dist
            self.backend = backend

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if not self.dist:
            return v
        import torch

        dev = f"cuda:{self.local}" if self.backend == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


# ----------------------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi samples during the timed region (every 200 ms)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


def workload_config(a) -> dict:
    return {"workload": f"incore BN cohort {a.n_ind} x {a.n_snp} (K=8 Dirichlet(1), Fst 0.02, p~U(.01,.5), "
                        f"2% missing), nrhs {a.nrhs}, one pass X^T X Omega per step",
            "n_ind": a.n_ind, "n_snp": a.n_snp, "nrhs": a.nrhs, "precision": a.precision,
            "packed_gb": round(a.n_snp * ((a.n_ind + 3) // 4) / 1e9, 3),
            "l2": "inputs larger than L2 (packed matrix >> 129 MB); no flush",
            "parallelism": "replicas (one independent solve per GPU)"}


# ----------------------------------------------------------------------------- reference arm
def reference_arm(a, ranks: Ranks) -> None:
    if ranks.rank != 0:
        return
    from distpca_gb300 import synth
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    c = synth.config_cohort("incore50k", n_snp=a.n_snp, n_ind=a.n_ind)
    S = min(a.cpu_snps, a.n_snp)
    sample = O.synth_rows(c, 0, S)
    om = O.omega(a.n_ind, a.nrhs)
    walls = []
    O.one_pass(sample, a.n_ind, om, bsize=min(10_000, S), npasses=a.warmup + a.steps, walls=walls)
    t = sum(walls[a.warmup:])
    value = a.n_ind * S * a.steps / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * t / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(a),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{S} SNPs x {a.n_ind} individuals per step (bsize 10000, steady-state "
                                       f"LUT passes), OpenBLAS {threads} threads, decode single-threaded as in "
                                       f"the reference"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- dpca arm
def dominant(kt: dict, prefer: tuple) -> str:
    cands = {k: v for k, v in kt.items() if v["launches"] > 0}
    for p in prefer:
        if p in cands:
            return max(((k, v) for k, v in cands.items() if k in prefer), key=lambda kv: kv[1]["ms"])[0]
    return max(cands.items(), key=lambda kv: kv[1]["ms"])[0]


def traffic_for(kernel: str, a):
    """DRAM bytes per launch from the committed ncu summary, if it covers this workload."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            d = json.load(f)
        w = d.get("workload", {})
        if (w.get("n_ind"), w.get("n_snp"), w.get("nrhs")) != (a.n_ind, a.n_snp, a.nrhs):
            return None
        return d.get(kernel)
    except Exception:
        return None


def dpca_arm(a, ranks: Ranks) -> None:
    import torch

    import distpca_gb300 as D
    from distpca_gb300 import synth

    dev = ranks.local
    torch.cuda.set_device(dev)
    # a dedicated (non-default) stream: the library launches on it and the events below time it
    stream = torch.cuda.Stream(device=dev)
    c = synth.config_cohort("incore50k", n_snp=a.n_snp, n_ind=a.n_ind)
    prec = D.PREC_MIXED if a.precision == "mixed" else D.PREC_FP64
    h = D.Handle(a.n_ind, a.n_snp, a.nrhs, precision=prec, device=dev, stream=stream.cuda_stream)
    h.reset_kernel_times(True)
    h.synth_fill(c)  # the device fill, then the per-SNP decode/statistics kernel over the resident matrix
    setup = h.kernel_times()
    omega = D.start_block(a.n_ind, a.nrhs)
    h.set_omega(omega)
    for _ in range(a.warmup):
        h.pass_()
    h.synchronize()
    h.reset_kernel_times(True)
    clocks = Clocks(dev)
    ranks.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        h.pass_()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    h.synchronize()  # raises if a bounded device wait gave up during the timed passes
    ranks.barrier()
    ms = e0.elapsed_time(e1)
    ms_max = ranks.max(ms)
    kt = h.kernel_times()
    h.reset_kernel_times(False)
    launches = int(sum(v["launches"] for v in kt.values()))
    value = a.n_ind * a.n_snp * a.steps * ranks.world / (ms_max / 1e3)
    pk = peaks()
    if a.precision == "mixed":
        dom = dominant(kt, ("mixed_xw", "mixed_xty"))
        flops = 2.0 * a.n_snp * a.n_ind * a.nrhs  # algorithmic flops of one product launch
        avg_s = kt[dom]["ms"] / kt[dom]["launches"] / 1e3
        roof = {"kernel": dom, "bound": "tensor", "achieved": flops / avg_s / 1e12,
                "peak": pk["bf16_tflops_sustained"], "unit": "TFLOP/s",
                "peak_source": f"{pk['source']} bf16 sustained (kernel timed inside a multi-pass loop)"}
        # the exact integer scheme issues two FP16 slices of the dense operand (N = 2 kp) for
        # each of the G' and M products: 4 x kp / k times the algorithmic MMA work
        kp = (a.nrhs + 7) // 8 * 8
        issued = flops * 4 * kp / a.nrhs
        roof["issued_tensor_flop_per_launch"] = issued
        roof["frac_issued"] = issued / avg_s / 1e12 / roof["peak"]
    else:
        dom = dominant(kt, ("fp64_xw", "fp64_xty"))
        flops = 2.0 * a.n_snp * a.n_ind * a.nrhs
        avg_s = kt[dom]["ms"] / kt[dom]["launches"] / 1e3
        roof = {"kernel": dom, "bound": "fp64", "achieved": flops / avg_s / 1e12, "peak": 1.25, "unit": "TFLOP/s",
                "peak_source": "nominal FP64 (no measured FP64 peak)"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["traffic"] = traffic_for(dom, a)
    roof["algorithmic_per_launch"] = f"{flops:.3e} flop (2 x n_snp x n_ind x nrhs)"
    kernels = {k: {"ms_per_launch": v["ms"] / max(1, v["launches"]), "launches": v["launches"],
                   "share": v["ms"] / max(1e-9, sum(x["ms"] for x in kt.values()))} for k, v in kt.items()}
    decode = None
    if "snp_stats" in setup and setup["snp_stats"]["launches"]:
        t_dec = setup["snp_stats"]["ms"] / setup["snp_stats"]["launches"] / 1e3
        packed_bytes = a.n_snp * ((a.n_ind + 3) // 4)
        decode = {"kernel": "snp_counts_kernel + snp_moments_kernel (decode, per-SNP counts, mean, sd, LUT)",
                  "ms": t_dec * 1e3,
                  "achieved_gbs": packed_bytes / t_dec / 1e9, "peak_gbs": pk["hbm_gbs"],
                  "frac": packed_bytes / t_dec / 1e9 / pk["hbm_gbs"], "bytes_per_launch": packed_bytes,
                  "note": "one launch per matrix (setup), timed with CUDA events on the handle's stream"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ranks.world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f16 hi+lo x exact 0/1/2, f32 accumulate, f64 dense" if a.precision ==
            "mixed" else "f64", "data": "synthetic (seeded Balding-Nichols, generated on the device)",
            "config": workload_config(a), "clocks": clk, "gpu_launches": launches, "roofline": roof, "decode": decode,
            "kernels": kernels}
    # ---- extras (rank 0, untimed): FP64 GPU comparison, accuracy, e2e, CPU baseline ----
    host = None
    np_bytes = (a.n_ind + 3) // 4
    if ranks.rank == 0 and not (a.no_e2e and a.no_cpu and a.no_extras):
        host = torch.empty((a.n_snp, np_bytes), dtype=torch.uint8, pin_memory=True)
        hv = host.numpy()
        D.lib().dpca_download_packed(h._h, 0, a.n_snp, hv.ctypes.data)
    h.close()
    torch.cuda.empty_cache()
    if ranks.rank == 0 and not a.no_extras and a.precision == "mixed":
        line["fp64_gpu"] = fp64_comparison(a, hv, value / ranks.world)
        line["accuracy"] = accuracy_check(a, hv)
    if ranks.rank == 0 and not a.no_e2e:
        line["e2e"] = e2e_run(a, hv)
    if ranks.rank == 0 and not a.no_extras:
        line["streamed"] = streamed_run(a, hv)
    if ranks.rank == 0 and not a.no_windows:
        line["windows"] = windows_run(a)
    if ranks.rank == 0 and not a.no_serve:
        line["serve"] = serve_run(a)
    if ranks.rank == 0 and not a.no_cpu and ranks.world == 1:
        line["cpu_baseline"] = cpu_baseline(a, hv)
    if ranks.rank == 0:
        print(json.dumps(line), flush=True)


def fp64_comparison(a, hv, mixed_per_gpu: float) -> dict:
    import torch

    import distpca_gb300 as D

    S = min(a.fp64_snps, a.n_snp)
    stream = torch.cuda.Stream()
    with D.Handle(a.n_ind, S, a.nrhs, precision=D.PREC_FP64, stream=stream.cuda_stream) as h:
        h.upload_ptr(hv.ctypes.data, hv.shape[1])
        h.set_omega(D.start_block(a.n_ind, a.nrhs))
        h.pass_()
        h.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2):
            h.pass_()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 2
    v = a.n_ind * S / (ms / 1e3)
    return {"value": v, "unit": UNIT, "sample": f"{S} SNPs x {a.n_ind} individuals, plain FP64 GPU path",
            "mixed_over_fp64": mixed_per_gpu / v}


def accuracy_check(a, hv) -> dict:
    """Mixed vs plain FP64 on the same start block, same fixed iteration count."""
    import distpca_gb300 as D

    S = min(a.accuracy_snps, a.n_snp)
    nsv = a.nrhs // 2
    sub = hv[:S]
    kw = dict(nsv=nsv, nrhs=a.nrhs, power=a.power, crit=1, tol=-1.0, miter=1, bsize=10_000, verbose=0)
    om = D.start_block(a.n_ind, a.nrhs)
    rm = D.run_packed(sub, a.n_ind, omega0=om, precision="mixed", **kw)
    rf = D.run_packed(sub, a.n_ind, omega0=om, precision="fp64", **kw)
    lam_m, lam_f = rm["sigma"] ** 2, rf["sigma"] ** 2
    qm, _ = np.linalg.qr(rm["u"])
    qf, _ = np.linalg.qr(rf["u"])
    s = np.clip(np.linalg.svd(qm.T @ qf, compute_uv=False), -1, 1)
    corr = np.abs(np.sum(rm["u"] * rf["u"], 0)) / (np.linalg.norm(rm["u"], axis=0) * np.linalg.norm(rf["u"], axis=0))
    return {"sample": f"{S} SNPs x {a.n_ind}, nrhs {a.nrhs}, nsv {nsv}, power {a.power}, 1 iteration",
            "eig_rel_err_max": float(np.max(np.abs(lam_m - lam_f) / lam_f)),
            "principal_angle_max_rad": float(np.arccos(s.min())),
            "pc_abs_corr_min": float(corr.min())}


def e2e_run(a, hv) -> dict:
    """Through the reference-facing C ABI (dpca_run_packed) from pinned host memory."""
    import distpca_gb300 as D

    kw = dict(nsv=a.nrhs // 2, nrhs=a.nrhs, power=a.power, crit=1, tol=-1.0, miter=1, bsize=10_000, verbose=0,
              precision=a.precision)
    om0 = D.start_block(a.n_ind, a.nrhs)
    D.run_packed(hv, a.n_ind, omega0=om0, **kw)  # warm-up (context, allocator)
    link = host_link_gbs(hv)
    times, passes, parts = [], 0, {}
    for _ in range(a.e2e_steps):
        t0 = time.perf_counter()
        r = D.run_packed(hv, a.n_ind, omega0=om0, **kw)
        times.append(time.perf_counter() - t0)
        passes = r["passes"]
        parts = {"load_s": r["time_load_matrix"], "products_s": r["time_mm"], "qr_s": r["time_gs"],
                 "rayleigh_ritz_s": r["time_projected_svd"], "other_s": r["time_other"], "streamed": r["streamed"]}
    t = sum(times) / len(times)
    return {"value": a.n_ind * a.n_snp * passes / t, "unit": UNIT,
            "h2d_bytes_per_step": int(hv.nbytes + a.n_ind * a.nrhs * 8),
            "d2h_bytes_per_step": int(a.n_ind * a.nrhs * 8),
            "call": f"dpca_run_packed, 1 outer iteration = {passes} passes incl. H2D, stats, QR, Rayleigh-Ritz",
            "seconds_per_call": t,
            "breakdown": parts,
            "host_link_gbs": link,
            "note": "the 12.5 GB host-to-device copy is part of each call; host_link_gbs is a plain pinned copy "
                    "measured just before (the host link is shared on this machine and varies between runs)"}


def host_link_gbs(hv) -> float:
    """Pinned host-to-device bandwidth of a plain 2 GB copy from the bench's host buffer."""
    import torch

    nbytes = min(hv.nbytes, 2_000_000_000)
    src = torch.from_numpy(hv.reshape(-1)[:nbytes])
    dst = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    dst.copy_(src, non_blocking=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        dst.copy_(src, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    del dst
    torch.cuda.empty_cache()
    return 3 * nbytes / (e0.elapsed_time(e1) / 1e3) / 1e9


def streamed_run(a, hv) -> dict:
    """The same pass with the rows streamed from pinned host memory in 2 GB blocks (the
    out-of-core block reader): genotypes/s and the host-to-device bandwidth it sustains."""
    import torch

    import distpca_gb300 as D

    np_bytes = hv.shape[1]
    pitch = (np_bytes + 127) // 128 * 128
    blk = max(128, (2_000_000_000 // pitch) // 128 * 128)
    stream = torch.cuda.Stream()
    prec = D.PREC_MIXED if a.precision == "mixed" else D.PREC_FP64
    with D.Handle(a.n_ind, a.n_snp, a.nrhs, precision=prec, stream=stream.cuda_stream, block_snps=blk) as h:
        h.upload(hv)
        h.set_omega(D.start_block(a.n_ind, a.nrhs))
        h.pass_()
        h.synchronize()
        steps = 2
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            h.pass_()
        e1.record(stream)
        torch.cuda.synchronize()
        h.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / steps
    return {"value": a.n_ind * a.n_snp / t, "unit": UNIT, "ms_per_pass": t * 1e3,
            "h2d_gbs": hv.nbytes / t / 1e9, "block_snps": blk, "blocks": (a.n_snp + blk - 1) // blk,
            "note": "rows in pinned host memory, two device blocks double-buffered on a copy stream"}


def windows_run(a) -> dict:
    """Batched local PCA: 4,096 SNP windows of log-uniform width in [500, 20,000] over a shared
    2,000-individual Balding-Nichols cohort (K = 4, Fst 0.05, 1% missing), nsv 2, nrhs 8, power 3,
    the reference's default convergence test (crit 1, tol 1e-3), solved together (dpca_windows_*,
    mixed precision).  Beside it, a sample of the same windows solved one at a time on their own
    handles (the first 16 windows)."""
    import distpca_gb300 as D
    from distpca_gb300 import synth

    n_ind = 2000
    widths = synth.window_widths(a.windows, seed=0)
    c = synth.make_cohort(n_ind, int(widths.sum()), n_pop=4, fst=0.05, missing=0.01, seed=4)
    flags = dict(nsv=2, power=3)
    with D.Windows(n_ind, widths, 8) as w:
        w.synth_fill(c)
        w.solve(miter=1, want_u=False, **flags)  # warm-up
        w.reset_kernel_times(True)
        t0 = time.perf_counter()
        r = w.solve(want_u=False, **flags)
        t = time.perf_counter() - t0
        kt = w.kernel_times()
    passes = (flags["power"] + 1) * r["its"]
    gpass = float(np.sum(widths * n_ind * passes))
    sample = min(16, a.windows)
    offs = np.concatenate([[0], np.cumsum(widths)])
    t1 = 0.0
    for i in range(sample):
        rows = synth.pack_rows(c, int(offs[i]), int(offs[i + 1]))
        t0 = time.perf_counter()
        with D.Handle(n_ind, int(widths[i]), 8, precision="mixed") as h:
            h.upload(rows)
            h.solve(D.start_block(n_ind, 8), bsize=int(widths[i]) - 1, **flags)
        t1 += time.perf_counter() - t0
    return {"windows": int(a.windows), "n_ind": n_ind, "snps": int(widths.sum()), "nrhs": 8, "nsv": 2, "power": 3,
            "seconds": t, "windows_per_s": a.windows / t, "genotype_passes_per_s": gpass / t,
            "its_mean": float(np.mean(r["its"])), "its_max": int(np.max(r["its"])),
            "kernel_ms": {k: round(v["ms"], 3) for k, v in kt.items()},
            "one_at_a_time": {"sample": f"the first {sample} windows, one handle each (create, upload, solve)",
                              "seconds": t1, "windows_per_s": sample / t1},
            "data": "seeded Balding-Nichols cohort filled on the device"}


def serve_run(a) -> dict:
    """The mixed-size job stream through the serving loop (dpca_serve_*): Poisson arrivals of
    seeded Balding-Nichols jobs (n_ind log-U[500, 20k], n_snp log-U[10k, 500k], nsv in {5, 10, 20},
    nrhs 2 nsv, power 4; the reference's defaults crit 1, tol 1e-3), each job's genotypes filled
    on the device.  Latency = completion - submission.  Beside it, jobs of the same stream run one
    at a time as plain FP64 GPU solves and as mixed solves (the first jobs of at most 2e8
    genotypes, which bounds the FP64 arm's time)."""
    import distpca_gb300 as D
    from distpca_gb300 import synth

    jobs = synth.serve_stream(a.serve_jobs, a.serve_rate, seed=0)
    cohorts = [synth.serve_cohort(j) for j in jobs]

    def flags(j, prec):
        return dict(nsv=j["nsv"], nrhs=j["nrhs"], power=j["power"], bsize=j["n_snp"], precision=prec)

    with D.Server(slots=a.serve_slots) as s:
        ids = []
        start = time.perf_counter()
        for j, c in zip(jobs, cohorts):
            d = start + j["t"] - time.perf_counter()
            if d > 0:
                time.sleep(d)
            ids.append(s.submit(j["n_ind"], j["n_snp"], cohort=c, want_u=False, **flags(j, "mixed")))
        res = [s.result(i) for i in ids]
        wall = time.perf_counter() - start
        st = s.stats()
    lat = np.array([r["info"].t_done - r["info"].t_submit for r in res])
    svc = np.array([r["info"].t_done - r["info"].t_start for r in res])
    gpass = sum(j["n_ind"] * j["n_snp"] * r["passes"] for j, r in zip(jobs, res))
    picked = [i for i, j in enumerate(jobs) if j["n_ind"] * j["n_snp"] <= 2e8][:a.serve_sample]

    def one_at_a_time(prec):
        with D.Server(slots=1) as s:
            out = []
            for i in picked:
                j = jobs[i]
                r = s.result(s.submit(j["n_ind"], j["n_snp"], cohort=cohorts[i], want_u=False, **flags(j, prec)))
                out.append(r["info"].t_done - r["info"].t_start)
        return float(sum(out))

    t64, tmx = one_at_a_time("fp64"), one_at_a_time("mixed")
    return {"jobs": len(jobs), "arrival_rate_per_s": a.serve_rate, "slots": a.serve_slots,
            "wall_s": wall, "jobs_per_s": len(jobs) / wall, "latency_p50_s": float(np.median(lat)),
            "latency_p99_s": float(np.quantile(lat, 0.99)), "service_p50_s": float(np.median(svc)),
            "genotype_passes_per_s": gpass / wall, "max_in_flight": st["max_in_flight"],
            "peak_device_gb": st["peak_gb"], "budget_gb": st["budget_gb"],
            "one_at_a_time": {"sample": f"jobs {picked} of the stream (the first {len(picked)} of <= 2e8 genotypes)",
                              "fp64_gpu_s": t64, "mixed_s": tmx, "fp64_jobs_per_s": len(picked) / t64,
                              "mixed_jobs_per_s": len(picked) / tmx},
            "data": "seeded Balding-Nichols cohorts filled on the device per job"}


def cpu_baseline(a, hv) -> dict:
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    S = min(a.cpu_snps, a.n_snp)
    om = O.omega(a.n_ind, a.nrhs)
    walls = []
    O.one_pass(np.ascontiguousarray(hv[:S]), a.n_ind, om, bsize=min(10_000, S), npasses=2, walls=walls)
    return {"value": a.n_ind * S / walls[-1], "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{S} SNPs x {a.n_ind} individuals, one steady-state pass (bsize 10000), OpenBLAS "
                      f"{threads} threads"}


def main():
    a = parse()
    ranks = Ranks()
    try:
        if a.impl == "reference":
            reference_arm(a, ranks)
        else:
            dpca_arm(a, ranks)
    finally:
        ranks.close()


if __name__ == "__main__":
    main()
