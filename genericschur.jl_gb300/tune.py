"""Tuner of the batched Schur kernels' launch shapes (run on the GPU it tunes for).

The persistent batched kernels (one CTA per matrix, a work queue per size bin) have a
launch shape per bin: the bin's largest order, threads per CTA, whether the Hessenberg
phase runs on a full copy of the matrix in shared memory, and a cap on CTAs per SM.
This script times every compiled shape on each bin's share of the benchmark batches --
20,000 real N(0,1) matrices with orders ~ U{8..128} (seed 4) and 5,000 complex ones
(seed 5) -- picks the fastest per bin, then tries a few bin boundaries with the chosen
shapes on the whole batch; for the FP32 stage of the mixed real form (GS_MIXED, default
bins kept) it improves one bin's shape at a time, largest bin first, timing the whole
mixed call on the real batch.  It writes the table that gs_set_tuning loads:

    python genericschur.jl_gb300/tune.py [--out PATH] [--reps 5] [--margin 0.02]

Timing: device-resident inputs, the launch sequence replayed as a CUDA graph (the
benchmark's mode), CUDA events around the library's kernels (gs_last_kernel_ms), median
of --reps runs after one warm-up run.  A shape replaces the hand-picked default only when
it is faster by --margin (the whole batch's run-to-run spread is about 1-2%).  A shape
whose results differ from the default shape's (status, or eigenvalues beyond 1e-8
relative) is never chosen.
"""
import argparse
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

THREADS = [64, 96, 128, 160, 192, 256]
DEFAULT_BOUNDS = [32, 64, 96, 128]
DEFAULT_THREADS = [64, 64, 128, 128]
DEFAULT_HSMEM = [1, 1, 0, 0]
BOUND_SETS = [[32, 64, 96, 128], [32, 64, 104, 128], [32, 72, 104, 128], [40, 72, 104, 128],
              [32, 64, 112, 128], [48, 80, 112, 128], [24, 56, 96, 128]]
MAX_DYN_SMEM = 227 * 1024 - 1024


def smem_bytes(kind, nmax, hsmem):
    """Dynamic shared memory per CTA, as the kernels size it."""
    if kind in ("real_f64", "mixed_f32"):
        full = nmax * (nmax | 1) if hsmem else 0
        rpk = (nmax * (nmax + 7)) // 2  # real packed QR layout: column j keeps rows 1..j+3
        return (8 if kind == "real_f64" else 4) * (max(full, rpk) + 6 * nmax + 32)
    pk = (nmax * (nmax + 5)) // 2  # complex packed QR layout: column j keeps rows 1..j+2
    h = nmax * (nmax | 1) if hsmem else pk
    return 16 * (h + 4 * nmax) + 32 * 8 + 64


def table_text(shapes, note):
    lines = ["# gschur_gb300 batched tuning table (genericschur.jl_gb300/tune.py)"]
    lines += ["# " + x for x in note]
    lines.append("# kind bin nmax threads hsmem ctas_per_sm")
    for kind in ("real_f64", "complex_f64", "mixed_f32"):
        for b, (nmax, nt, hs, ctas) in enumerate(shapes[kind]):
            lines.append("%s %d %d %d %d %d" % (kind, b, nmax, nt, hs, ctas))
    return "\n".join(lines) + "\n"


class Runner:
    """Device-resident copy of one batch and a timed call of the batched entry point."""

    def __init__(self, ctx, torch, dev, kind, packed, ns, offs, woffs, mixed=False):
        from genericschur_gb300 import _capi
        self.ctx, self.torch, self.kind, self.count = ctx, torch, kind, len(ns)
        self.cplx = kind == "complex_f64"
        data = packed.view(np.float64) if self.cplx else packed
        self.A0 = torch.from_numpy(np.ascontiguousarray(data)).to(dev)
        self.A = torch.empty_like(self.A0)
        self.Z = torch.empty_like(self.A0)
        nw = int(ns.sum())
        self.w1 = torch.empty(2 * nw if self.cplx else nw, dtype=torch.float64, device=dev)
        self.w2 = torch.empty(nw, dtype=torch.float64, device=dev)
        self.st = torch.empty(len(ns), dtype=torch.int32, device=dev)
        self.ns, self.offs, self.woffs = (torch.from_numpy(x).to(dev) for x in (ns, offs, woffs))
        # the benchmark's mode: the launch sequence replayed as a CUDA graph
        self.flags = _capi.GS_WANTZ | _capi.GS_SCALE | _capi.GS_DEVICE | _capi.GS_GRAPH
        if mixed:
            self.flags |= _capi.GS_MIXED
        self.stream = torch.cuda.Stream(dev)

    def run(self):
        lib, h = self.ctx.lib, self.ctx.handle
        self.A.copy_(self.A0)
        self.torch.cuda.synchronize()
        self.ctx.set_stream(self.stream.cuda_stream)
        try:
            if self.cplx:
                rc = lib.gs_schur_batched_c64(h, self.count, self.ns.data_ptr(), self.offs.data_ptr(),
                                              self.woffs.data_ptr(), self.A.data_ptr(), self.Z.data_ptr(),
                                              self.w1.data_ptr(), self.st.data_ptr(), self.flags)
            else:
                rc = lib.gs_schur_batched_f64(h, self.count, self.ns.data_ptr(), self.offs.data_ptr(),
                                              self.woffs.data_ptr(), self.A.data_ptr(), self.Z.data_ptr(),
                                              self.w1.data_ptr(), self.w2.data_ptr(), self.st.data_ptr(),
                                              self.flags)
            self.stream.synchronize()
        finally:
            self.ctx.set_stream(None)
        if rc != 0:
            raise RuntimeError(self.ctx.last_error())
        return self.ctx.last_kernel_ms()

    def eigenvalues(self):
        w = self.w1.cpu().numpy()
        w = w.view(np.complex128) if self.cplx else w + 1j * self.w2.cpu().numpy()
        return w, int((self.st != 0).sum().item())

    def time(self, reps):
        self.run()
        return float(np.median([self.run() for _ in range(reps)]))


def apply(ctx, shapes, tmpdir):
    path = os.path.join(tmpdir, "candidate.tsv")
    with open(path, "w") as f:
        f.write(table_text(shapes, []))
    ctx.set_tuning(path)


def close_enough(w, w_ref):
    a = np.sort_complex(w)
    b = np.sort_complex(w_ref)
    return bool(np.all(np.abs(a - b) <= 1e-8 * np.maximum(1.0, np.abs(b))))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "genericschur_gb300", "tuning", "sm_103a.tsv"))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--margin", type=float, default=0.02,
                    help="a shape replaces the default only when it is faster by this fraction")
    args = ap.parse_args()
    import torch
    import build_lib
    build_lib.build()
    import genericschur_gb300 as gs
    from genericschur_gb300.workloads import batched_cplx, batched_real
    dev = torch.device("cuda", 0)
    os.environ["GS_TUNING"] = ""  # start from the built-in shapes
    ctx = gs.Context(0)
    t_start = time.time()
    base_shapes = [(b, nt, hs, 0) for b, nt, hs in zip(DEFAULT_BOUNDS, DEFAULT_THREADS, DEFAULT_HSMEM)]
    default = {"real_f64": list(base_shapes), "complex_f64": list(base_shapes), "mixed_f32": list(base_shapes)}
    batches = {"real_f64": batched_real(20000, seed=4), "complex_f64": batched_cplx(5000, seed=5)}
    chosen = {k: list(v) for k, v in default.items()}
    log = []
    with tempfile.TemporaryDirectory() as tmp:
        for kind in ("real_f64", "complex_f64"):
            packed, ns, offs, woffs = batches[kind]
            lo = 0
            for b, hi in enumerate(DEFAULT_BOUNDS):
                sel = np.nonzero((ns > lo) & (ns <= hi))[0]
                blo, lo = lo + 1, hi
                sub = gs.pack_batch([packed[offs[i]:offs[i] + ns[i] ** 2].reshape(ns[i], ns[i], order="F")
                                     for i in sel], np.complex128 if kind == "complex_f64" else np.float64)
                r = Runner(ctx, torch, dev, kind, *sub)
                apply(ctx, default, tmp)
                base_ms = r.time(args.reps)
                w_ref, bad = r.eigenvalues()
                assert bad == 0
                best = (base_ms, default[kind][b])
                for nt in THREADS:
                    for hs in (0, 1):
                        if smem_bytes(kind, hi, hs) > MAX_DYN_SMEM:
                            continue
                        cand = {k: list(v) for k, v in default.items()}
                        cand[kind][b] = (hi, nt, hs, 0)
                        apply(ctx, cand, tmp)
                        ms = r.time(args.reps)
                        w, bad = r.eigenvalues()
                        ok = bad == 0 and close_enough(w, w_ref)
                        log.append("%s bin %d (n %d..%d, %d matrices) threads %d hsmem %d: %.2f ms%s"
                                   % (kind, b, blo, hi, len(sel), nt, hs, ms, "" if ok else " REJECTED"))
                        print(log[-1], flush=True)
                        if ok and ms < best[0] and ms < base_ms * (1.0 - args.margin):
                            best = (ms, (hi, nt, hs, 0))
                chosen[kind][b] = best[1]
                del r
                torch.cuda.empty_cache()
            # bin boundaries with the chosen shapes (the shape of the default bin holding each bound)
            r = Runner(ctx, torch, dev, kind, *batches[kind])
            apply(ctx, default, tmp)
            base = r.time(args.reps)
            best = None
            for bounds in BOUND_SETS:
                cand = {k: list(v) for k, v in chosen.items()}
                shapes = []
                for b, hi in enumerate(bounds):
                    src = next(i for i, d in enumerate(DEFAULT_BOUNDS) if hi <= d)
                    _, nt, hs, ctas = chosen[kind][src]
                    if smem_bytes(kind, hi, hs) > MAX_DYN_SMEM:
                        hs = 0
                    shapes.append((hi, nt, hs, ctas))
                cand[kind] = shapes
                apply(ctx, cand, tmp)
                ms = r.time(args.reps)
                _, bad = r.eigenvalues()
                log.append("%s whole batch, bounds %s: %.2f ms%s" % (kind, bounds, ms, "" if bad == 0 else " REJECTED"))
                print(log[-1], flush=True)
                if bad == 0 and (best is None or ms < best[0]):
                    best = (ms, shapes)
            # keep the hand-picked shapes unless the winner beats them by the margin
            if best is None or best[0] > base * (1.0 - args.margin):
                best = (base, default[kind])
            chosen[kind] = best[1]
            log.append("%s whole batch: default shapes %.2f ms, chosen %.2f ms" % (kind, base, best[0]))
            print(log[-1], flush=True)
            del r
            torch.cuda.empty_cache()
        # FP32 stage of the mixed form: one bin at a time on the whole mixed call
        r = Runner(ctx, torch, dev, "real_f64", *batches["real_f64"], mixed=True)
        apply(ctx, chosen, tmp)
        base = cur = r.time(args.reps)
        _, bad = r.eigenvalues()
        assert bad == 0
        for b in reversed(range(len(DEFAULT_BOUNDS))):
            hi = DEFAULT_BOUNDS[b]
            for nt in THREADS:
                for hs in (0, 1):
                    if nt == 160 or smem_bytes("mixed_f32", hi, hs) > MAX_DYN_SMEM or \
                            (hi, nt, hs, 0) == chosen["mixed_f32"][b]:
                        continue
                    cand = {k: list(v) for k, v in chosen.items()}
                    cand["mixed_f32"][b] = (hi, nt, hs, 0)
                    apply(ctx, cand, tmp)
                    ms = r.time(args.reps)
                    _, bad = r.eigenvalues()
                    log.append("mixed_f32 bin %d threads %d hsmem %d: whole mixed batch %.2f ms%s"
                               % (b, nt, hs, ms, "" if bad == 0 else " REJECTED"))
                    print(log[-1], flush=True)
                    if bad == 0 and ms < cur * (1.0 - args.margin):
                        cur = ms
                        chosen["mixed_f32"][b] = (hi, nt, hs, 0)
        log.append("mixed_f32 whole mixed batch: default shapes %.2f ms, chosen %.2f ms" % (base, cur))
        print(log[-1], flush=True)
        del r
        torch.cuda.empty_cache()
    note = ["device: %s; tuned %s in %.0f s" % (torch.cuda.get_device_name(0), time.strftime("%Y-%m-%d"),
                                                 time.time() - t_start),
            "workloads: real 20000 N(0,1) n~U{8..128} seed 4; complex 5000 seed 5; CUDA graph replay; "
            "a shape replaces the default only when %.0f%% faster" % (100 * args.margin)] + \
        [x for x in log if "whole batch" in x or "whole mixed batch: default" in x]
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    with open(args.out, "w") as f:
        f.write(table_text(chosen, note))
    print(open(args.out).read())


if __name__ == "__main__":
    main()
