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
    p.add_argument("--serve-stable-jobs", type=int, default=256,
                   help="jobs in the second stream, offered at 80%% of the capacity the first one measured")
    p.add_argument("--no-full", action="store_true", help="skip the whole-PCA legs (config 1, converged config 2)")
    p.add_argument("--no-tune", action="store_true", help="skip the autotuner (heuristic launch parameters)")
    p.add_argument("--no-ooc", action="store_true", help="skip the 500,000-individual out-of-core stream")
    p.add_argument("--ooc-snps", type=int, default=2_000_000, help="SNPs of the out-of-core stream")
    p.add_argument("--ooc-distinct", type=int, default=4, help="distinct 2 GB blocks cycled by the out-of-core source")
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
    tune = None
    if a.precision == "mixed" and not a.no_tune:
        tune = h.autotune()  # once per shape class, before the timed region
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
        # the exact integer scheme issues two FP16 slices of the dense operand (N = 2 kp) for the
        # G' product (and, in the two-product kernel, again for the M product): 2 x kp / k (4 x)
        # times the algorithmic MMA work
        kern = (tune or {}).get("kernel") or ("gprod" if os.environ.get("DPCA_MIXED_KERNEL") == "gprod"
                                             else "products")
        kp = (a.nrhs + 7) // 8 * 8
        issued = flops * (4 if kern == "products" else 2) * kp / a.nrhs
        roof["mixed_kernel"] = kern
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
            "kernels": kernels, "autotune": tune}
    # ---- extras (rank 0, untimed): FP64 GPU comparison, accuracy, e2e, CPU baseline ----
    host = hv = None
    np_bytes = (a.n_ind + 3) // 4
    if ranks.rank == 0 and not (a.no_e2e and a.no_extras and a.no_full):
        host = torch.empty((a.n_snp, np_bytes), dtype=torch.uint8, pin_memory=True)
        hv = host.numpy()
        D.lib().dpca_download_packed(h._h, 0, a.n_snp, hv.ctypes.data)
    h.close()
    torch.cuda.empty_cache()
    if hv is not None and not a.no_extras and a.precision == "mixed":
        line["fp64_gpu"] = fp64_comparison(a, hv, value / ranks.world)
        line["accuracy"] = accuracy_check(a, hv)
    if hv is not None and not a.no_e2e:
        line["e2e"] = e2e_run(a, hv)
    if hv is not None and not a.no_full and a.precision == "mixed":
        line["full_pca"] = {"incore50k_converged": converged_run(a, hv)}
    if hv is not None and not a.no_extras:
        line["streamed"] = streamed_run(a, hv)
    del hv, host
    if ranks.rank == 0 and not a.no_full and a.precision == "mixed":
        line.setdefault("full_pca", {})["config1_1k_x_100k"] = config1_run(a)
    if ranks.rank == 0 and not a.no_ooc and a.precision == "mixed":
        line["out_of_core"] = out_of_core_run(a)
    if ranks.rank == 0 and not a.no_windows:
        line["windows"] = windows_run(a)
    if ranks.rank == 0 and not a.no_serve:
        sat = serve_run(a, a.serve_rate, a.serve_jobs, compare=True)
        if not a.no_tune:
            sat["tuned"] = serve_tune(a)
            tuned = serve_run(a, a.serve_rate, a.serve_jobs, compare=False)
            sat["tuned"].update({k: tuned[k] for k in ("jobs_per_s", "latency_p50_s", "latency_p99_s",
                                                       "service_p50_s", "service_p99_s", "wall_s")})
        # capacity: the same jobs offered all at once (the 50/s stream is arrival-bound once the
        # loop keeps up with it); the stable-load stream is offered at 80% of that
        cap = serve_run(a, 1e6, a.serve_jobs, compare=False)
        sat["capacity"] = {k: cap[k] for k in ("jobs_per_s", "wall_s", "latency_p50_s", "latency_p99_s",
                                               "service_p50_s", "service_p99_s", "genotype_passes_per_s",
                                               "max_in_flight", "peak_device_gb")}
        sat["capacity"]["offered"] = f"the same {a.serve_jobs} jobs submitted at once"
        stable_rate = round(0.8 * cap["jobs_per_s"], 1)
        sat["stable_load"] = serve_run(a, stable_rate, a.serve_stable_jobs, compare=False)
        line["serve"] = sat
    if ranks.rank == 0 and not a.no_cpu and ranks.world == 1:
        line["cpu_baseline"] = cpu_baseline_rows(a)
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


def host_link_gbs(hv, nbytes: int = 2_000_000_000) -> float:
    """Host-to-device bandwidth of plain copies (cudaMemcpyAsync, through torch) of the first
    `nbytes` of the bench's own pinned host buffer -- the memory the timed copies read."""
    import torch

    nbytes = min(hv.nbytes, nbytes)
    src = torch.from_numpy(hv.reshape(-1)[:nbytes])
    dst = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        dst.copy_(src, non_blocking=True)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        e1.record(stream)
    stream.synchronize()
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
    link0 = host_link_gbs(hv)
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
    link1 = host_link_gbs(hv)
    gbs = hv.nbytes / t / 1e9
    return {"value": a.n_ind * a.n_snp / t, "unit": UNIT, "ms_per_pass": t * 1e3,
            "h2d_gbs": gbs, "link_gbs_before_after": [link0, link1], "frac_of_link": gbs / max(link0, link1),
            "block_snps": blk, "blocks": (a.n_snp + blk - 1) // blk,
            "note": "the in-core matrix's rows in pinned host memory, streamed in ~2 GB blocks every pass; the "
                    "link is measured with cudaMemcpyAsync from the same pinned buffer just before and after"}


def converged_run(a, hv) -> dict:
    """Wall time of whole PCAs of the in-core matrix through dpca_run_packed (pinned host rows,
    the host-to-device copy inside), run to convergence: with the published runs' flags (crit 2,
    tol 1e-3) and with the reference's code defaults (crit 1, tol 1e-3); nsv 20, nrhs 40, power 6,
    bsize 10,000 (the out-of-core variant of the solver)."""
    import distpca_gb300 as D

    om0 = D.start_block(a.n_ind, a.nrhs)
    out = {}
    for name, crit in (("crit2_tol1e-3", 2), ("crit1_tol1e-3", 1)):
        kw = dict(nsv=a.nrhs // 2, nrhs=a.nrhs, power=a.power, crit=crit, tol=1e-3, miter=100, bsize=10_000,
                  verbose=0, precision="mixed")
        t0 = time.perf_counter()
        r = D.run_packed(hv, a.n_ind, omega0=om0, **kw)
        t = time.perf_counter() - t0
        out[name] = {"seconds": t, "its": r["its"], "passes": r["passes"],
                     "genotype_passes_per_s": a.n_ind * a.n_snp * r["passes"] / t,
                     "load_s": r["time_load_matrix"], "sigma_1": float(r["sigma"][0])}
    return out


def config1_run(a) -> dict:
    """The 1,000 x 100,000 workload the reference runs on a CPU (Balding-Nichols K = 5 x 200,
    Fst 0.05, p ~ U(0.05, 0.5), 1% missing, seed 0; nsv 10, nrhs 20, power 4, tol 1e-6, bsize
    10,000): the whole PCA through dpca_run_packed from pinned host rows, in both precisions, and
    the CPU restatement of the reference on all host cores for three outer iterations, scaled to
    the iterations the FP64 run took (the full CPU run takes minutes)."""
    import torch

    import distpca_gb300 as D
    from distpca_gb300 import synth

    n_ind, n_snp = 1000, 100_000
    c = synth.make_cohort(n_ind, n_snp, n_pop=5, pop_sizes=[200] * 5, fst=0.05, p_range=(0.05, 0.5), missing=0.01,
                          seed=0)
    host = torch.empty((n_snp, (n_ind + 3) // 4), dtype=torch.uint8, pin_memory=True)
    hv = host.numpy()
    with D.Handle(n_ind, n_snp, 1, precision="fp64") as h:
        h.synth_fill(c)
        D.lib().dpca_download_packed(h._h, 0, n_snp, hv.ctypes.data)
    kw = dict(nsv=10, nrhs=20, power=4, crit=1, tol=1e-6, miter=100, bsize=10_000, verbose=0)
    om0 = D.start_block(n_ind, 20)
    out = {"workload": "1000 x 100000, nsv 10, nrhs 20, power 4, crit 1, tol 1e-6, bsize 10000"}
    for prec in ("mixed", "fp64"):
        D.run_packed(hv, n_ind, omega0=om0, miter=1, **{k: v for k, v in kw.items() if k != "miter"},
                     precision=prec)  # warm-up
        t0 = time.perf_counter()
        r = D.run_packed(hv, n_ind, omega0=om0, precision=prec, **kw)
        t = time.perf_counter() - t0
        out[prec] = {"seconds_per_pca": t, "its": r["its"], "passes": r["passes"],
                     "genotype_passes_per_s": n_ind * n_snp * r["passes"] / t}
    if not a.no_cpu:
        from oracle import oracle as O

        threads = os.cpu_count() or 1
        O.set_threads(threads)
        t0 = time.perf_counter()
        O.solve(hv, n_ind, nsv=10, nrhs=20, power=4, crit=1, tol=-1.0, miter=3, bsize=10_000, omega0=om0)
        t3 = time.perf_counter() - t0
        its = out["fp64"]["its"]
        out["cpu_reference_port"] = {"seconds_3_iterations": t3, "seconds_per_pca_estimate": t3 / 3 * its,
                                     "cores": threads, "kind": "port",
                                     "note": f"3 outer iterations timed, scaled to the {its} iterations of the run"}
        out["fp64_speedup_vs_cpu"] = out["cpu_reference_port"]["seconds_per_pca_estimate"] / out["fp64"]["seconds_per_pca"]
        out["mixed_speedup_vs_cpu"] = out["cpu_reference_port"]["seconds_per_pca_estimate"] / out["mixed"]["seconds_per_pca"]
    return out


def out_of_core_run(a) -> dict:
    """The out-of-core shape: 500,000 individuals x `ooc_snps` SNPs (250 GB packed at 2,000,000,
    more than this machine's host memory), nrhs 20, mixed precision, streamed from pinned host memory
    in ~2 GB SNP blocks every pass.  The rows come from a block source (dpca_upload_blocks) that
    cycles over `ooc_distinct` distinct ~2 GB blocks of a seeded Balding-Nichols cohort (K = 10,
    Fst 0.01, p ~ Beta(0.5, 2) clipped to [0.005, 0.5], 5% missing in 10% of the samples): a
    matrix whose SNP blocks repeat, which costs the stream and the products exactly what distinct
    blocks would.  The host link is measured with cudaMemcpyAsync from the same pinned blocks
    just before and after the timed passes."""
    import torch

    import distpca_gb300 as D
    from distpca_gb300 import synth

    n_ind, n_snp, k = 500_000, a.ooc_snps, 20
    npb = (n_ind + 3) // 4
    pitch = (npb + 127) // 128 * 128
    blk = max(128, (2_000_000_000 // pitch) // 128 * 128)
    dist = max(1, min(a.ooc_distinct, (n_snp + blk - 1) // blk))
    c = synth.make_cohort(n_ind, dist * blk, n_pop=10, fst=0.01, p_beta=(0.5, 2.0), p_clip=(0.005, 0.5),
                          missing=0.05, heavy_frac=0.1, heavy_rate=0.05, seed=3)
    host = torch.empty((dist * blk, npb), dtype=torch.uint8, pin_memory=True)
    hv = host.numpy()
    with D.Handle(n_ind, dist * blk, 1, precision="fp64") as h:
        h.synth_fill(c)
        D.lib().dpca_download_packed(h._h, 0, dist * blk, hv.ctypes.data)
    torch.cuda.empty_cache()
    base = hv.ctypes.data

    def rows(s0, n):
        j = (s0 // blk) % dist
        return base + j * blk * npb, npb

    link0 = host_link_gbs(hv)
    stream = torch.cuda.Stream()
    with D.Handle(n_ind, n_snp, k, precision="mixed", stream=stream.cuda_stream, block_snps=blk) as h:
        h.upload_blocks(rows, max_row_stride=npb)  # the statistics sweep reads every block once
        h.set_omega(D.start_block(n_ind, k))
        h.pass_()
        h.synchronize()
        h.reset_kernel_times(True)
        steps = 2
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            h.pass_()
        e1.record(stream)
        torch.cuda.synchronize()
        h.synchronize()
        kt = h.kernel_times()
        t = e0.elapsed_time(e1) / 1e3 / steps
    link1 = host_link_gbs(hv)
    packed_bytes = n_snp * npb
    gbs = packed_bytes / t / 1e9
    return {"n_ind": n_ind, "n_snp": n_snp, "nrhs": k, "packed_gb": packed_bytes / 1e9, "value": n_ind * n_snp / t,
            "unit": UNIT, "seconds_per_pass": t, "h2d_gbs": gbs, "link_gbs_before_after": [link0, link1],
            "frac_of_link": gbs / max(link0, link1), "block_snps": blk, "blocks": (n_snp + blk - 1) // blk,
            "distinct_blocks": dist,
            "kernel_ms_per_pass": {kk: round(v["ms"] / steps, 2) for kk, v in kt.items()},
            "note": "every pass copies all packed rows host-to-device (two device blocks, copy stream beside the "
                    "compute stream); the kernel times overlap the copies"}


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


def serve_run(a, rate: float, n_jobs: int, compare: bool) -> dict:
    """The mixed-size job stream through the serving loop (dpca_serve_*): Poisson arrivals of
    seeded Balding-Nichols jobs (n_ind log-U[500, 20k], n_snp log-U[10k, 500k], nsv in {5, 10, 20},
    nrhs 2 nsv, power 4; the reference's defaults crit 1, tol 1e-3), each job's genotypes filled
    on the device.  Latency = completion - submission.  Beside it, jobs of the same stream run one
    at a time as plain FP64 GPU solves and as mixed solves (the first jobs of at most 2e8
    genotypes, which bounds the FP64 arm's time)."""
    import distpca_gb300 as D
    from distpca_gb300 import synth

    jobs = synth.serve_stream(n_jobs, rate, seed=0)
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

    out = {"jobs": len(jobs), "arrival_rate_per_s": rate, "slots": a.serve_slots, "last_arrival_s": jobs[-1]["t"],
           "wall_s": wall, "jobs_per_s": len(jobs) / wall, "latency_p50_s": float(np.median(lat)),
           "latency_p99_s": float(np.quantile(lat, 0.99)), "service_p50_s": float(np.median(svc)),
           "service_p99_s": float(np.quantile(svc, 0.99)),
           "genotype_passes_per_s": gpass / wall, "max_in_flight": st["max_in_flight"],
           "peak_device_gb": st["peak_gb"], "budget_gb": st["budget_gb"],
           "data": "seeded Balding-Nichols cohorts filled on the device per job"}
    if compare:
        t64, tmx = one_at_a_time("fp64"), one_at_a_time("mixed")
        out["one_at_a_time"] = {"sample": f"jobs {picked} of the stream (the first {len(picked)} of <= 2e8 genotypes)",
                                "fp64_gpu_s": t64, "mixed_s": tmx, "fp64_jobs_per_s": len(picked) / t64,
                                "mixed_jobs_per_s": len(picked) / tmx}
    return out


def serve_tune(a, classes: int = 12) -> dict:
    """Autotune the shape classes (individual tiles, SNP blocks and padded nrhs, one octave each)
    that the serving stream's jobs fall in most often, each on one representative job's matrix;
    the serving loop's handles of those classes start from the tuned choice."""
    import math

    import distpca_gb300 as D
    from distpca_gb300 import synth

    def octv(v):
        return 0 if v <= 1 else math.ceil(math.log2(v))

    jobs = synth.serve_stream(a.serve_jobs, a.serve_rate, seed=0)
    groups = {}
    for j in jobs:
        key = (octv(-(-j["n_ind"] // 128)), octv(-(-j["n_snp"] // 64)), (j["nrhs"] + 7) // 8 * 8)
        groups.setdefault(key, []).append(j)
    top = sorted(groups.items(), key=lambda kv: -len(kv[1]))[:classes]
    t0 = time.perf_counter()
    reports = []
    for key, js in top:
        j = js[0]
        with D.Handle(j["n_ind"], j["n_snp"], j["nrhs"], precision="mixed") as h:
            h.synth_fill(synth.serve_cohort(j))
            h.set_omega(D.start_block(j["n_ind"], j["nrhs"]))
            r = h.autotune()
        reports.append({"class": list(key), "jobs": len(js), "n_ind": j["n_ind"], "n_snp": j["n_snp"],
                        "nrhs": j["nrhs"], **r})
    return {"classes_tuned": len(top), "jobs_covered": sum(len(js) for _, js in top), "tuning_s":
            time.perf_counter() - t0, "per_class": reports}


def cpu_baseline_rows(a) -> dict:
    from distpca_gb300 import synth
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    S = min(a.cpu_snps, a.n_snp)
    c = synth.config_cohort("incore50k", n_snp=a.n_snp, n_ind=a.n_ind)
    sample = O.synth_rows(c, 0, S)  # the first S rows of the same matrix
    om = O.omega(a.n_ind, a.nrhs)
    walls = []
    O.one_pass(sample, a.n_ind, om, bsize=min(10_000, S), npasses=2, walls=walls)
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
