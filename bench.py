"""Benchmark of the batched real Float64 Schur decomposition (the headline workload).

Workload: 20,000 real Float64 matrices, orders iid uniform in [8, 128], entries iid
N(0,1), seed 4 (one batch per rank); each step is one gschur! over the whole batch
returning T, Z and the eigenvalues at FP64 backward error.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The metric compares the mixed form with the FP64 form at equal backward error: the
headline `value` is the mixed form (GS_MIXED: FP32 Schur sweeps, FP64 Newton refinement
of each Schur pair, FP64 recomputation of the matrices the refinement cannot finish),
`fp64` the plain FP64 batched form on the same inputs, and `accuracy` both forms'
backward and orthogonality errors on the same sample.  `value` is matrices/s with the
inputs resident in HBM (CUDA events on the launch stream; the step includes restoring
A, which the decomposition overwrites); `e2e` is the same metric through the C-ABI with
pinned host buffers, host<->device copies inside the timed region.  `--impl reference`
times the CPU restatement of the reference algorithm (the oracle, FP64) on the host
cores instead.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "genericschur.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "batched Schur matrices/s & n=4096 Schur time: mixed vs FP64, same backward err"
UNIT = "matrices/s"
COUNT, SEED = 20000, 4
WORKLOAD = "batched real FP64 Schur (T, Z, eigenvalues): 20000 matrices, n~U{8..128}, N(0,1), seed 4"


def bench_config(count):
    """The workload's config object, identical in both arms."""
    return {"workload": WORKLOAD, "batch": count, "seed": SEED,
            "l2": "inputs larger than L2 (%.0f MB of A per step); A restored from a pristine copy each step"
                  % (8e-6 * float(np.sum(np.asarray(_sizes(count), dtype=np.float64) ** 2)))}


def _sizes(count):
    from genericschur_gb300.workloads import batch_sizes
    return batch_sizes(count, SEED)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--count", type=int, default=COUNT)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="plain stream launches instead of the CUDA graph")
    ap.add_argument("--no-large", action="store_true", help="skip the n=4096 FP64 vs mixed-precision timing")
    ap.add_argument("--large-n", type=int, default=4096)
    ap.add_argument("--large-only", action="store_true",
                    help="only the large-matrix measurement (for profiling runs); prints its JSON object")
    ap.add_argument("--large-mode", default="both", choices=["both", "fp64", "mixed"])
    ap.add_argument("--gemm-only", action="store_true",
                    help="only the FP64 product on the BF16 tensor cores vs cuBLAS DGEMM; prints its JSON object")
    ap.add_argument("--gemm-n", type=int, default=4096)
    ap.add_argument("--dc-only", action="store_true",
                    help="only the divide-and-conquer tridiagonal eigensolver (n = --dc-n); prints its JSON object")
    ap.add_argument("--dc-n", type=int, default=4096)
    ap.add_argument("--gcond-only", action="store_true",
                    help="only the generalized condition estimates of a complex triangular pair (n = --gcond-n, "
                         "split in half); prints its JSON object")
    ap.add_argument("--gcond-n", type=int, default=1200)
    ap.add_argument("--case", choices=["mixed_once", "refine_small", "complex256"],
                    help="profiling cases (no timing, no JSON line): mixed_once = two GS_MIXED calls on the headline "
                         "batch (device buffers); refine_small = one GS_MIXED call on 600 matrices of orders 97..128; "
                         "complex256 = two plain complex Schur decompositions of the 256 x 256 workload")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def rank_seed(rank):
    """Each rank factors its own batch (weak scaling, no data-path collective)."""
    return SEED + rank


def reduce_max_ms(torch, ms, world, device):
    """The per-step time as the job sees it: the maximum over ranks."""
    if world <= 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, count, ms):
    """Matrices per second of the whole job: every rank's batch over the slowest rank's step."""
    return world * count / (ms * 1e-3)


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops(torch, dev):
    """Measured FP64 peak: cuBLAS DGEMM 4096^3 (best of 5), the FP64 analogue of the
    driver's cuBLAS bf16 figure."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * 4096.0 ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def fp32_peak_tflops(torch, dev):
    """Measured FP32 CUDA-core peak: cuBLAS SGEMM 4096^3 with TF32 off (best of 5)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(4096, 4096, dtype=torch.float32, device=dev)
        b = torch.randn(4096, 4096, dtype=torch.float32, device=dev)
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            best = max(best, 2 * 4096.0 ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
        del a, b
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return best


def measured_traffic_per_matrix():
    """DRAM bytes per matrix of the batched kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_schur_real_traffic.txt")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_matrix"):
                return float(line.split()[1])
    except OSError:
        pass
    return None


def cpu_baseline_sample(count, seed, budget_s=15.0):
    """Oracle (C++ restatement of the reference algorithm), OpenMP over the batch on
    all host cores, on a bounded sample of the same workload."""
    from oracle import pyoracle as po
    from genericschur_gb300.workloads import batched_real
    threads = os.cpu_count() or 1
    # calibrate on a small sample, then size the sample for ~budget_s
    pk, ns, offs, woffs = batched_real(count=64, seed=seed + 1000)
    t = time.perf_counter()
    _run_oracle(po, pk, ns, offs, woffs, threads)
    dt = max(time.perf_counter() - t, 1e-3)
    m = int(min(count, max(64, 64 * budget_s / dt)))
    pk, ns, offs, woffs = batched_real(count=m, seed=seed)
    t = time.perf_counter()
    bad = _run_oracle(po, pk, ns, offs, woffs, threads)
    dt = time.perf_counter() - t
    return {"value": m / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "first %d matrices of the seed-%d batch (same size law), %d failed" % (m, seed, bad),
            "seconds": dt}


def _run_oracle(po, pk, ns, offs, woffs, threads):
    a = pk.copy()
    z = np.zeros_like(a)
    nw = int(ns.sum())
    wr = np.zeros(nw)
    wi = np.zeros(nw)
    st = np.zeros(len(ns), dtype=np.int32)
    return po.gschur_batched_packed_real(len(ns), offs, ns, a, z, wr, wi, woffs, st, threads)


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import build as ob
    ob.build()
    samples = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline_sample(args.count, SEED, budget_s=8.0)
        if i >= args.warmup:
            samples.append(r)
    v = float(np.mean([s["value"] for s in samples]))
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": float(np.mean([s["seconds"] for s in samples]) * 1e3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": bench_config(args.count),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": samples[0]["cores"], "kind": "port",
                            "sample": samples[0]["sample"] + "; C++ restatement of GenericSchur.jl's gschur! "
                                      "(Julia is absent on this machine), OpenMP over the batch"},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_ours(args):
    import torch
    import build_lib
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build_lib.build()
    import genericschur_gb300 as gs
    from genericschur_gb300 import _capi
    from genericschur_gb300.workloads import batched_real, real_flops

    ctx = gs.Context(local)
    packed, ns, offs, woffs = batched_real(count=args.count, seed=rank_seed(rank))
    nw = int(ns.sum())
    count = len(ns)
    flops = real_flops(ns)
    # device-resident buffers
    dA0 = torch.from_numpy(packed).to(dev)
    dA = torch.empty_like(dA0)
    dZ = torch.empty_like(dA0)
    dwr = torch.empty(nw, dtype=torch.float64, device=dev)
    dwi = torch.empty(nw, dtype=torch.float64, device=dev)
    dns = torch.from_numpy(ns).to(dev)
    doffs = torch.from_numpy(offs).to(dev)
    dwoffs = torch.from_numpy(woffs).to(dev)
    dst = torch.empty(count, dtype=torch.int32, device=dev)
    # a dedicated (non-default) stream: the library and the CUDA events share it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    base_flags = _capi.GS_WANTZ | _capi.GS_SCALE | _capi.GS_DEVICE | (0 if args.no_graph else _capi.GS_GRAPH)
    lib = ctx.lib

    def make_step(flags):
        def step():
            dA.copy_(dA0)
            rc = lib.gs_schur_batched_f64(ctx.handle, count, dns.data_ptr(), doffs.data_ptr(), dwoffs.data_ptr(),
                                          dA.data_ptr(), dZ.data_ptr(), dwr.data_ptr(), dwi.data_ptr(),
                                          dst.data_ptr(), flags)
            if rc != 0:
                raise RuntimeError("gs_schur_batched_f64 failed: %s" % ctx.last_error())
        return step

    def timed(flags, sample_clocks):
        """W warm-up steps, then K steps between a barrier and synchronizes (CUDA events on
        the library's stream); returns ms per step, the kernel-only ms of two further
        steps, unconverged count, the clock record, and the results of the last step."""
        step = make_step(flags)
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        bad = int((dst != 0).sum().item())
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local) if sample_clocks else None
        if clocks:
            clocks.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ms_total = e0.elapsed_time(e1)
        clk = clocks.stop() if clocks else None
        kms = []
        for _ in range(2):
            step()
            torch.cuda.synchronize()
            kms.append(ctx.last_kernel_ms())
        res = (dA.cpu().numpy(), dZ.cpu().numpy(), dwr.cpu().numpy() + 1j * dwi.cpu().numpy())
        return ms_total / args.steps, float(np.mean(kms)), bad, clk, res

    # headline: the mixed form (FP32 Schur sweeps, FP64 Newton refinement; FP64 accuracy)
    mixed_flags = base_flags | _capi.GS_MIXED
    ms_mixed, kms_mixed, bad, clk, res_mixed = timed(mixed_flags, True)
    info = ctx.mixed_info()  # counters and refinement time of the last (kernel-timed) step
    # the plain FP64 batched form on the same inputs
    ms_fp64, kms_fp64, bad64, _, res_fp64 = timed(base_flags, False)
    ms = reduce_max_ms(torch, ms_mixed, world, dev)
    value = job_throughput(world, count, ms)
    value64 = job_throughput(world, count, reduce_max_ms(torch, ms_fp64, world, dev))

    e2e = e2e64 = None
    if not args.no_e2e:
        e2e = measure_e2e(ctx, packed, ns, offs, woffs, steps=max(1, min(args.steps, 3)), mixed=True)
        e2e64 = measure_e2e(ctx, packed, ns, offs, woffs, steps=max(1, min(args.steps, 3)))
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    peak = fp64_peak_tflops(torch, dev)
    peak32 = fp32_peak_tflops(torch, dev)
    # roofline of the mixed step's dominant kernel: the FP32 batched Schur kernel
    # (k_schur_real<float>, four size-bin launches running concurrently), timed by the CUDA
    # events the library records at the start of the call's kernels and at the start of the
    # refinement (the conversion k_mixed_prep, ~1% of the stage, is inside that window);
    # bound by the FP32 FMA pipe (25 n^3 FLOP per matrix), which the bulge chase's
    # dependent chains and per-step barriers leave mostly idle
    fp32_s = info["fp32_us"] * 1e-6 if info["fp32_us"] > 0 else None
    ach32 = flops / fp32_s / 1e12 if fp32_s else None
    roof = {"bound": "fp32", "achieved": ach32, "peak": peak32, "unit": "TFLOP/s",
            "frac": (ach32 / peak32) if ach32 else None, "traffic": None,
            "kernel": "k_schur_real<float> (FP32 stage of the mixed step, four size-bin launches)",
            "phase_ms": info["fp32_us"] * 1e-3, "step_kernel_ms": kms_mixed,
            "algorithmic": "25 n^3 FP32 FLOP per matrix, summed over the batch (%.4g FLOP per launch)" % flops,
            "peak_source": "measured: cuBLAS SGEMM 4096^3 in this run (FP32 FMA pipe, TF32 off)",
            "traffic_note": "not the bound: inputs and outputs are 12 n^2 bytes per matrix (ncu: "
                            "profiles/k_schur_real_f32_600.md)"}
    # the refinement phase: FP64-accurate products on the tensor cores, the rest of each
    # Newton step in FP32; its rate in FP64-equivalent FLOPs of those products
    ref_s = info["refine_us"] * 1e-6 if info["refine_us"] > 0 else None
    refinement = dict(info)
    refinement.update({
        "phase_ms": info["refine_us"] * 1e-3,
        "product_fp64_equiv_tflops": info["product_flops"] / ref_s / 1e12 if ref_s else None,
        "fp64_peak_tflops": peak,
        "kernels": "k_refine_tc (tensor cores: A_s Z, Z^T (A Z), Z^T Z per Newton step), k_refine_bin<2,4,6,8> "
                   "(FP32 Sylvester waves, corrections), one launch each per Newton step (six steps)",
        "algorithmic": "per Newton step 2 n^3 each for A_s Z, Z^T (A_s Z), Z^T Z; %.4g FLOP in %d Newton steps "
                       "over %d matrices" % (info["product_flops"], info["newton_steps"],
                                             info["refined"] + info["handed_back"])})
    kernel_ms = kms_fp64
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    per_matrix_bytes = measured_traffic_per_matrix()
    traffic = per_matrix_bytes * count if per_matrix_bytes else None
    roof64 = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
              "traffic": traffic, "kernel": "k_schur_real<double> (four size-bin launches)",
              "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of the 4 size-bin launches of one "
                                "step, ncu capture of a 6000-matrix case of the same law scaled by matrices "
                                "(profiles/k_schur_real_traffic.txt); algorithmic bytes 24 n^2 + 16 n per matrix "
                                "= %.4g per step" % float(np.sum(24.0 * ns.astype(np.float64) ** 2 + 16.0 * ns)),
              "algorithmic": "25 n^3 FLOP per matrix, summed over the batch (%.4g FLOP per launch)" % flops,
              "kernel_ms": kernel_ms}
    accuracy = {"mixed": schur_errors_sample(packed, ns, offs, woffs, res_mixed),
                "fp64": schur_errors_sample(packed, ns, offs, woffs, res_fp64)}
    fp64 = {"value": value64, "unit": UNIT, "ms_per_step": ms_fp64, "unconverged": bad64, "roofline": roof64,
            "e2e": e2e64, "gpu_launches_per_step": 5}
    cpu = None if args.no_cpu else cpu_baseline_sample(args.count, SEED)
    per_matrix = measure_per_matrix(ctx, packed, ns, offs)
    secondary = measure_complex_and_adjoint(ctx, torch, dev, stream)
    large = None
    large_small = None
    precision = None
    c1 = None
    gemm_tc = None
    stedc = None
    if not args.no_large:
        ctx.set_stream(None)
        large = measure_large(ctx, torch, dev, args.large_n)
        large_small = [measure_large(ctx, torch, dev, m) for m in (1024, 2048)]
        precision = measure_precision(ctx, torch, dev)
        c1 = measure_c1(ctx)
        gemm_tc = measure_gemm_tc(ctx, torch, dev, args.large_n)
        stedc = measure_stedc(ctx, args.dc_n)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
           "form": "mixed (GS_MIXED): FP32 Schur sweeps, per-matrix Newton refinement of the Schur pair with its "
                   "FP64-accurate products on the BF16 tensor cores, FP64 recomputation of matrices the refinement "
                   "cannot finish; results at FP64 backward error (accuracy: both forms measured on the same "
                   "sample in this run)",
           "config": bench_config(args.count), "graph": not args.no_graph,
           "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
           "gpu_launches": 42 * args.steps, "unconverged": bad, "refinement": refinement,
           "fp64": fp64, "mixed_vs_fp64": value / value64,
           "mixed_vs_fp64_e2e": (e2e["value"] / e2e64["value"]) if (e2e and e2e64) else None,
           "accuracy": accuracy, "plain_fp64_per_matrix": per_matrix,
           "large": large, "large_1024_2048": large_small, "precision": precision, "complex256": c1,
           "gemm_f64_tc": gemm_tc, "stedc": stedc, **secondary}
    print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def measure_large(ctx, torch, dev, n, mode="both"):
    """The second half of the metric: one n x n real Schur decomposition (iid N(0,1),
    seed 1 for n=4096) by the plain FP64 path and by the FP32 + FP64-refinement path,
    each through the C-ABI with host buffers (copies included), with its backward
    error ||A - Z T Z^T||_F / ||A||_F and orthogonality ||Z^T Z - I||_F in units of
    n eps (computed on the GPU in FP64 after the timed call)."""
    import ctypes
    import genericschur_gb300 as gs
    from genericschur_gb300.workloads import large_real, LARGE_SEEDS
    A = large_real(n)
    eps = np.finfo(np.float64).eps
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).to(dev).T  # column-major view

    def errors(S):
        T = torch.from_numpy(np.ascontiguousarray(S.T.T)).to(dev).T
        Z = torch.from_numpy(np.ascontiguousarray(S.Z.T)).to(dev).T
        be = torch.linalg.norm(dA - Z @ T @ Z.T) / torch.linalg.norm(dA)
        oe = torch.linalg.norm(Z.T @ Z - torch.eye(n, dtype=torch.float64, device=dev))
        return float(be) / (n * eps), float(oe) / (n * eps)

    out = {"n": n, "seed": LARGE_SEEDS.get(n, n), "entries": "iid N(0,1)"}
    if mode in ("both", "fp64"):
        t = time.perf_counter()
        S = gs.gschur(A, ctx=ctx)
        out["fp64_s"] = time.perf_counter() - t
        out["fp64_kernel_ms"] = ctx.last_kernel_ms()
        out["fp64_backward_err_n_eps"], out["fp64_orth_err_n_eps"] = errors(S)
    if mode in ("both", "mixed"):
        t = time.perf_counter()
        S, info = gs.gschur_mixed(A, ctx=ctx, return_info=True)
        out["mixed_s"] = time.perf_counter() - t
        out["mixed_kernel_ms"] = ctx.last_kernel_ms()
        out["mixed_backward_err_n_eps"], out["mixed_orth_err_n_eps"] = errors(S)
        out["mixed_refinement"] = info
    if mode == "both":
        out["speedup_mixed_vs_fp64"] = out["fp64_s"] / out["mixed_s"]
    out["flops_25n3"] = 25.0 * n ** 3
    return out


def _schur_errors(torch, dev, A, S):
    """||A - Z T Z^T||_F / ||A||_F and ||Z^T Z - I||_F in units of n eps (FP64 on the GPU)."""
    n = A.shape[0]
    eps = np.finfo(np.float64).eps
    cm = lambda M: torch.from_numpy(np.ascontiguousarray(M)).to(dev)
    dA, T, Z = cm(A), cm(S.T), cm(S.Z)
    be = torch.linalg.norm(dA - Z @ T @ Z.T) / torch.linalg.norm(dA)
    oe = torch.linalg.norm(Z.T @ Z - torch.eye(n, dtype=torch.float64, device=dev))
    return float(be) / (n * eps), float(oe) / (n * eps)


def measure_precision(ctx, torch, dev, n=2048):
    """The precision workload's own matrix: A = V diag(l) V^-1, l real with |l| log-uniform
    in [1e-3, 1e3] and random signs, cond(V) = 1e3, seed 6, n = 2048.  The plain FP64 path
    and the FP32 + FP64-refinement entry point, each through the C-ABI with host buffers,
    with their backward errors.  On this law FP32's own backward error (eps32 ||A||_F ~
    0.07) exceeds half of the eigenvalues' gaps, so the refinement has nothing to converge
    to and the entry point recomputes in FP64 (info iterations = -1); the line records
    what that costs."""
    import genericschur_gb300 as gs
    from genericschur_gb300.workloads import conditioned_matrix
    A = conditioned_matrix(n, seed=6)
    t = time.perf_counter()
    S = gs.gschur(A, ctx=ctx)
    fp64_s = time.perf_counter() - t
    be64, oe64 = _schur_errors(torch, dev, A, S)
    t = time.perf_counter()
    S2, info = gs.gschur_mixed(A, ctx=ctx, return_info=True)
    mixed_s = time.perf_counter() - t
    be, oe = _schur_errors(torch, dev, A, S2)
    return {"workload": "A = V diag(l) V^-1, n=2048, |l| log-uniform [1e-3,1e3], random signs, cond(V)=1e3, seed 6",
            "norm_fro": float(np.linalg.norm(A)), "fp64_s": fp64_s, "fp64_backward_err_n_eps": be64,
            "fp64_orth_err_n_eps": oe64, "mixed_s": mixed_s, "mixed_backward_err_n_eps": be,
            "mixed_orth_err_n_eps": oe, "mixed_info": info,
            "note": "iterations -1: FP64 recomputation (FP32 cannot separate this law's eigenvalues)"}


def measure_c1(ctx, n=256):
    """The plain CPU-runnable workload: one 256 x 256 ComplexF64 matrix, re/im iid
    N(0, 1/2), seed 0, Z accumulated, no balancing.  GPU time of gs_schur_c64 (host
    buffers, median of 3 after a warm-up) beside the oracle (the C++ restatement of the
    reference's complex gschur!, one core) on the same matrix."""
    import genericschur_gb300 as gs
    from oracle import pyoracle as po
    rng = np.random.default_rng(0)
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2)
    ts = []
    for _ in range(4):
        t = time.perf_counter()
        S = gs.gschur(A, ctx=ctx)
        ts.append(time.perf_counter() - t)
    gpu_s = float(np.median(ts[1:]))
    kernel_ms = ctx.last_kernel_ms()
    t = time.perf_counter()
    po.gschur(A)
    cpu_s = time.perf_counter() - t
    eps = np.finfo(np.float64).eps
    be = np.linalg.norm(A - S.Z @ S.T @ S.Z.conj().T) / np.linalg.norm(A) / (n * eps)
    return {"workload": "256x256 ComplexF64, re/im N(0,1/2), seed 0, Z accumulated", "gpu_s": gpu_s,
            "gpu_kernel_ms": kernel_ms, "cpu_oracle_s": cpu_s, "cpu_oracle_cores": 1,
            "backward_err_n_eps": float(be), "flops_100n3": 100.0 * n ** 3}


def measure_per_matrix(ctx, packed, ns, offs, sample=200):
    """The plain FP64 path one matrix per call (gs_schur_f64 with device buffers,
    synchronised per call) on the first `sample` matrices of the batch: what a caller
    without the batched form gets, for comparison with the persistent batched launch."""
    import torch
    from genericschur_gb300 import _capi
    dev = torch.device("cuda", torch.cuda.current_device())
    m = min(sample, len(ns))
    mats = [torch.from_numpy(packed[offs[b]:offs[b] + int(ns[b]) ** 2].copy()).to(dev) for b in range(m)]
    Z = torch.empty(128 * 128, dtype=torch.float64, device=dev)
    wr = torch.empty(128, dtype=torch.float64, device=dev)
    wi = torch.empty(128, dtype=torch.float64, device=dev)
    flags = _capi.GS_WANTZ | _capi.GS_SCALE | _capi.GS_DEVICE
    torch.cuda.synchronize()
    t = time.perf_counter()
    for b in range(m):
        n = int(ns[b])
        rc = ctx.lib.gs_schur_f64(ctx.handle, n, mats[b].data_ptr(), n, Z.data_ptr(), n, wr.data_ptr(), wi.data_ptr(),
                                  flags, 0)
        if rc not in (0, 1):
            raise RuntimeError(ctx.last_error())
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    return {"value": m / dt, "unit": UNIT, "sample": "first %d matrices of the batch, one gs_schur_f64 call each "
            "(device buffers)" % m}


def measure_complex_and_adjoint(ctx, torch, dev, stream, steps=3):
    """Secondary configs on device-resident inputs, CUDA events on the library's stream:
    (a) gschur! over 5,000 ComplexF64 matrices, n ~ U{8..128}, seed 5 (one persistent
    launch sequence); (b) the differentiation workload -- 4,096 complex 64 x 64 matrices,
    seed 7: forward Schur + eigenvalue adjoint (eigenvectors recomputed from T, Z) per step."""
    from genericschur_gb300 import _capi
    from genericschur_gb300.workloads import adjoint_batch, batched_cplx, cplx_flops, logsumexp_loss
    out = {}
    # the library must launch on the stream the events are recorded on
    ctx.set_stream(stream.cuda_stream)

    def timed(fn, k):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    for name, (packed, ns, offs, woffs) in (("complex_batched", batched_cplx(5000, seed=5)),
                                            ("adjoint", adjoint_batch(4096, 64, seed=7))):
        cnt = len(ns)
        A0 = torch.from_numpy(packed.view(np.float64)).to(dev)
        A = torch.empty_like(A0)
        Z = torch.empty_like(A0)
        w = torch.empty(2 * int(ns.sum()), dtype=torch.float64, device=dev)
        st = torch.empty(cnt, dtype=torch.int32, device=dev)
        dns = torch.from_numpy(ns).to(dev)
        doffs = torch.from_numpy(offs).to(dev)
        dwoffs = torch.from_numpy(woffs).to(dev)
        flags = _capi.GS_WANTZ | _capi.GS_SCALE | _capi.GS_DEVICE | _capi.GS_GRAPH

        def fwd():
            A.copy_(A0)
            rc = ctx.lib.gs_schur_batched_c64(ctx.handle, cnt, dns.data_ptr(), doffs.data_ptr(), dwoffs.data_ptr(),
                                              A.data_ptr(), Z.data_ptr(), w.data_ptr(), st.data_ptr(), flags)
            if rc != 0:
                raise RuntimeError(ctx.last_error())

        if name == "complex_batched":
            ms = timed(fwd, steps)
            out[name] = {"value": cnt / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
                         "workload": "5000 ComplexF64 matrices, n~U{8..128}, re/im N(0,1/2), seed 5",
                         "tflops_100n3": cplx_flops(ns) / (ms * 1e-3) / 1e12}
        else:
            fwd()
            torch.cuda.synchronize()
            _, gbar = logsumexp_loss(torch.view_as_complex(w.view(-1, 2)).cpu().numpy(), woffs, 64)
            dg = torch.from_numpy(gbar.view(np.float64)).to(dev)
            G = torch.empty_like(A0)
            plen, wlen = len(packed), int(ns.sum())

            def step():
                fwd()
                rc = ctx.lib.gs_eig_adjoint_batched_c64(ctx.handle, cnt, dns.data_ptr(), doffs.data_ptr(),
                                                        dwoffs.data_ptr(), plen, wlen, A.data_ptr(), Z.data_ptr(),
                                                        dg.data_ptr(), G.data_ptr(), _capi.GS_DEVICE)
                if rc != 0:
                    raise RuntimeError(ctx.last_error())

            ms = timed(step, steps)
            out[name] = {"value": cnt / (ms * 1e-3), "unit": "matrices/s (forward Schur + eigenvalue adjoint)",
                         "ms_per_step": ms,
                         "workload": "4096 ComplexF64 64x64, entries complex N(0,1/2)/8, seed 7, "
                                     "loss sum logsumexp(Re(l)/0.1)"}
    ctx.set_stream(None)
    return out


def schur_errors_sample(packed, ns, offs, woffs, res, every=20):
    """Backward error ||A - Z T Z^T||_F / ||A||_F and orthogonality ||Z^T Z - I||_F, in
    units of n eps, of every `every`-th matrix of a batch result (numpy, on the host)."""
    T, Z, _ = res
    be, oe = [], []
    for b in range(0, len(ns), every):
        n = int(ns[b])
        o = int(offs[b])
        A = packed[o:o + n * n].reshape((n, n), order="F")
        Tb = T[o:o + n * n].reshape((n, n), order="F")
        Zb = Z[o:o + n * n].reshape((n, n), order="F")
        eps = np.finfo(np.float64).eps
        be.append(np.linalg.norm(A - Zb @ Tb @ Zb.T) / np.linalg.norm(A) / (n * eps))
        oe.append(np.linalg.norm(Zb.T @ Zb - np.eye(n)) / (n * eps))
    return {"backward_max": float(np.max(be)), "backward_median": float(np.median(be)),
            "orth_max": float(np.max(oe)), "orth_median": float(np.median(oe)), "unit": "n eps",
            "sample": "every %dth matrix (%d)" % (every, len(be))}


def measure_e2e(ctx, packed, ns, offs, woffs, steps, mixed=False):
    """Same metric through the C-ABI with pinned host buffers (copies included)."""
    import ctypes
    from genericschur_gb300 import _capi
    count = len(ns)
    nw = int(ns.sum())
    nbytes = packed.nbytes
    hp = [ctx.host_alloc(nbytes) for _ in range(2)]
    hw = [ctx.host_alloc(nw * 8) for _ in range(2)]
    hs = ctx.host_alloc(count * 4)
    try:
        A = np.ctypeslib.as_array((ctypes.c_double * packed.size).from_address(hp[0]))
        Z = np.ctypeslib.as_array((ctypes.c_double * packed.size).from_address(hp[1]))
        ctx.set_stream(None)
        flags = _capi.GS_WANTZ | _capi.GS_SCALE | (_capi.GS_MIXED if mixed else 0)
        times = []
        for i in range(steps + 1):
            A[:] = packed
            t = time.perf_counter()
            rc = ctx.lib.gs_schur_batched_f64(ctx.handle, count, ns.ctypes.data, offs.ctypes.data,
                                              woffs.ctypes.data, hp[0], hp[1], hw[0], hw[1], hs, flags)
            dt = time.perf_counter() - t
            if rc != 0:
                raise RuntimeError(ctx.last_error())
            if i > 0:
                times.append(dt)
        dt = float(np.mean(times))
        h2d = nbytes + ns.nbytes + offs.nbytes + woffs.nbytes
        d2h = 2 * nbytes + 2 * nw * 8 + count * 4
        return {"value": count / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "seconds_per_step": dt, "seconds_samples": [round(x, 4) for x in times],
                "kernel_ms_last": ctx.last_kernel_ms()}
    finally:
        for p in hp + hw + [hs]:
            ctx.host_free(p)


def measure_gemm_tc(ctx, torch, dev, n, reps=5):
    """The refinement's FP64 product on the BF16 tensor cores (gs_gemm_f64_tc, exact
    splitting) against cuBLAS DGEMM on the FP64 pipe: C = A^T B, n x n x n, device
    buffers, CUDA events around the library's launches (split + product).  Tensor work
    per launch: 55 slice products x 2 n^3 BF16 FLOP."""
    from genericschur_gb300 import _capi
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    A = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    B = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    C = torch.empty(n, n, dtype=torch.float64, device=dev)
    ctx.set_stream(None)
    ms = []
    for i in range(3 + reps):
        rc = ctx.lib.gs_gemm_f64_tc(ctx.handle, n, n, n, A.data_ptr(), n, 1, B.data_ptr(), n, C.data_ptr(), n,
                                    _capi.GS_DEVICE)
        if rc != 0:
            raise RuntimeError(ctx.last_error())
        if i >= 3:
            ms.append(ctx.last_kernel_ms())
    tc_ms = float(np.median(ms))
    # column-major C = A_cm^T B_cm is, in torch's row-major view, C^T = A B^T
    ref = A @ B.T
    err = float((C.T - ref).norm() / ref.norm())
    torch.cuda.synchronize()
    dg = []
    for i in range(3 + reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(A, B)
        e1.record()
        e1.synchronize()
        if i >= 3:
            dg.append(e0.elapsed_time(e1))
    dgemm_ms = float(np.median(dg))
    peak = None
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"]
    except (OSError, KeyError, ValueError):
        peak = None
    tensor_tflops = 55 * 2.0 * n ** 3 / (tc_ms * 1e-3) / 1e12
    return {"n": n, "tc_ms": tc_ms, "dgemm_ms": dgemm_ms, "speedup_vs_dgemm": dgemm_ms / tc_ms,
            "fp64_equiv_tflops": 2.0 * n ** 3 / (tc_ms * 1e-3) / 1e12, "bf16_tensor_tflops": tensor_tflops,
            "bf16_peak_tflops": peak, "frac_of_bf16_peak": (tensor_tflops / peak) if peak else None,
            "rel_err_vs_dgemm": err}


def measure_stedc(ctx, n, reps=3):
    """_gschur!(SymTridiagonal(d, e), DivideAndConquer(), Z = I) through the C-ABI on a
    seeded random tridiagonal of order n (N(0,1) diagonal and off-diagonal): device time of
    the call (its events bracket the whole tree, host-side index work included), the
    eigenvalue error against LAPACK's tridiagonal solver and the orthogonality of Z."""
    import scipy.linalg
    import genericschur_gb300 as gs
    rng = np.random.default_rng(21)
    D, E = rng.standard_normal(n), rng.standard_normal(n - 1)
    times = []
    for _ in range(reps + 1):
        d, _, Z = gs.gschur_symtridiag(gs.SymTridiagonal(D.copy(), E.copy()), np.eye(n), alg="DivideAndConquer",
                                       ctx=ctx)
        times.append(ctx.last_kernel_ms())
    times = times[1:]
    ref = scipy.linalg.eigh_tridiagonal(D, E, eigvals_only=True)
    nT = max(np.abs(D).max(), np.abs(E).max()) * 3
    eps = np.finfo(float).eps
    ev_err = float(np.abs(np.sort(d) - ref).max() / (n * eps * nT))
    orth = float(np.abs(Z.T @ Z - np.eye(n)).max() / (n * eps))
    return {"n": n, "seed": 21, "entries": "d, e iid N(0,1)", "ms_min": float(min(times)),
            "ms_median": float(np.median(times)), "eigenvalue_err_n_eps_T": ev_err, "orth_err_n_eps": orth}


def measure_gcond(ctx, n, reps=3):
    """eigvalscond / subspacesep of a seeded random complex triangular pair (S, T), n x n,
    split in half (the generalized Sylvester wavefront of gcondition.cu): device times."""
    import genericschur_gb300 as gs
    rng = np.random.default_rng(7600)
    cn = lambda: (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2)
    S = np.triu(cn(), 1) / np.sqrt(n) + np.diag(cn()[0])
    T = np.triu(cn(), 1) / np.sqrt(n) + np.diag(1 + 0.5 * rng.random(n))
    G = gs.GeneralizedSchur(S, T, np.diag(S), np.diag(T), np.eye(n), np.eye(n))
    k = n // 2
    te, ts = [], []
    for _ in range(reps + 1):
        pl, pr = gs.eigvalscond(G, k, ctx=ctx)
        te.append(ctx.last_kernel_ms())
        sep = gs.subspacesep(G, k, ctx=ctx)
        ts.append(ctx.last_kernel_ms())
    return {"n": n, "nsub": k, "eigvalscond_ms": float(min(te[1:])), "subspacesep_ms": float(min(ts[1:])),
            "pl": float(pl), "pr": float(pr), "sep": [float(x) for x in sep]}


def run_gcond_only(args):
    import torch
    import build_lib
    torch.cuda.set_device(0)
    build_lib.build()
    import genericschur_gb300 as gs
    ctx = gs.Context(0)
    print(json.dumps(measure_gcond(ctx, args.gcond_n)))


def run_dc_only(args):
    import torch
    import build_lib
    torch.cuda.set_device(0)
    build_lib.build()
    import genericschur_gb300 as gs
    ctx = gs.Context(0)
    print(json.dumps(measure_stedc(ctx, args.dc_n)))


def run_gemm_only(args):
    import torch
    import build_lib
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    build_lib.build()
    import genericschur_gb300 as gs
    ctx = gs.Context(0)
    print(json.dumps(measure_gemm_tc(ctx, torch, dev, args.gemm_n)))


def run_large_only(args):
    import torch
    import build_lib
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    build_lib.build()
    import genericschur_gb300 as gs
    ctx = gs.Context(0)
    print(json.dumps(measure_large(ctx, torch, dev, args.large_n, args.large_mode)))


def run_case(args):
    """Small fixed cases for ncu launch lists and captures (profiles/)."""
    import torch
    import build_lib
    build_lib.build()
    import genericschur_gb300 as gs
    from genericschur_gb300 import _capi
    if args.case == "complex256":
        rng = np.random.default_rng(0)
        A = (rng.standard_normal((256, 256)) + 1j * rng.standard_normal((256, 256))) / np.sqrt(2)
        for _ in range(2):
            gs.gschur(A)
        return
    if args.case == "refine_small":
        rng = np.random.default_rng(12)
        mats = [rng.standard_normal((int(n), int(n))) for n in rng.integers(97, 129, size=600)]
        _, _, _, st = gs.gschur_batched(mats, mixed=True)
        assert np.all(st == 0)
        return
    from genericschur_gb300.workloads import batched_real
    dev = torch.device("cuda", 0)
    ctx = gs.Context(0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    packed, ns, offs, woffs = batched_real(count=COUNT, seed=SEED)
    dA = torch.from_numpy(packed).to(dev)
    dZ = torch.empty_like(dA)
    nw = int(ns.sum())
    dwr = torch.empty(nw, dtype=torch.float64, device=dev)
    dwi = torch.empty_like(dwr)
    dns, doffs, dwo = (torch.from_numpy(x).to(dev) for x in (ns, offs, woffs))
    dst = torch.empty(len(ns), dtype=torch.int32, device=dev)
    flags = _capi.GS_WANTZ | _capi.GS_SCALE | _capi.GS_DEVICE | _capi.GS_MIXED
    for _ in range(2):
        dA.copy_(torch.from_numpy(packed).to(dev))
        rc = ctx.lib.gs_schur_batched_f64(ctx.handle, len(ns), dns.data_ptr(), doffs.data_ptr(), dwo.data_ptr(),
                                          dA.data_ptr(), dZ.data_ptr(), dwr.data_ptr(), dwi.data_ptr(),
                                          dst.data_ptr(), flags)
        if rc != 0:
            raise RuntimeError(ctx.last_error())
    torch.cuda.synchronize()
    assert int((dst != 0).sum()) == 0


def main():
    args = parse()
    if args.case:
        run_case(args)
        return
    if args.large_only:
        run_large_only(args)
        return
    if args.gemm_only:
        run_gemm_only(args)
        return
    if args.dc_only:
        run_dc_only(args)
        return
    if args.gcond_only:
        run_gcond_only(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
