"""Benchmark: Sternheimer solves/sec on the production-size system.

Workload (one "step"): every right-hand side of the 8-atom simple-cubic
system (a = 10.26 bohr, 25 Ry, 40^3 FFT box, 2293 plane waves at k+q,
32 Kleinman-Bylander projectors, 16 occupied bands, 113 perturbations
Delta V = exp(i(q+G).r)) solved for 35 complex frequencies (+-omega: 70 shifts)
to the absolute seed residual 1e-10 with BiCGStab(4): 1808 right-hand sides,
126,560 (RHS, shift) solves per step.  One solve = one converged
(right-hand side, shift) pair.

Arms:
  default           the GB300 library (libsgw_gb300.so) through its C ABI;
                    ``value`` times the kernels with inputs resident in HBM,
                    ``e2e`` the same call with pinned host buffers (copies in).
  --impl reference  the reference algorithm on the host CPU: the C
                    restatement of bicgstab.f90 (oracle/), OpenMP over
                    right-hand sides, on a bounded sample of the same workload.
Run ``python bench.py`` (1 GPU) or under torchrun for N replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LMAX = 4
THRESHOLD = 1e-10
METRIC = "Sternheimer solves/sec: batched mixed vs plain FP64, same GPU, W err ≤1e-6"
WORKLOAD = "sc8 a=10.26 25Ry 40^3 npw=2293 nkb=32 nocc=16 npert=113 nfreq=35 (S=70) lmax=4 thr=1e-10"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def make_workload():
    from sternheimergw_gb300 import linter, synth
    t = time.time()
    s, f = synth.config("c1")
    nocc = s["nocc"]
    npert = len(s["gpert"])
    bb = np.zeros((npert * nocc, s["npw"]), dtype=np.complex128)
    for ip in range(npert):
        bb[ip * nocc:(ip + 1) * nocc] = linter.coulomb_rhs(s, ip)
    sh1 = linter.coulomb_shifts(s, f)
    sigma = np.tile(sh1, (npert, 1))
    log(f"[bench] workload built in {time.time() - t:.1f}s: nrhs={bb.shape[0]} S={sigma.shape[1]} npw={s['npw']}")
    return s, f, bb, sigma


# --- algorithmic FP64 work of one solve --------------------------------------
def flops_per_apply(s, op_shape):
    """FP64 flops of one H apply of this (pruned) algorithm: 5 M log2 M per
    FFT line actually needed, V_loc(r) multiply, projector and P_v contractions,
    kinetic + sigma."""
    nr1, nr2, nr3 = [int(v) for v in s["nr"]]
    ncol, ni1 = op_shape
    line = lambda m: 5.0 * m * math.log2(m)
    fft = 2 * (ncol * line(nr3) + ni1 * nr3 * line(nr2) + nr2 * nr3 * line(nr1))
    n = s["npw"]
    nkb = s["vkb"].shape[1]
    nocc = s["evq"].shape[1]
    return fft + 2.0 * nr1 * nr2 * nr3 + 16.0 * n * (nkb + nocc) + 14.0 * n


def column_shape(s):
    nr1, nr2 = int(s["nr"][0]), int(s["nr"][1])
    b = np.asarray(s["nl"])
    i1 = b % nr1
    i2 = (b // nr1) % nr2
    cols = set(zip(i1.tolist(), i2.tolist()))
    return len(cols), len(set(i1.tolist()))


def step_flops(s, iters, nshift, lmax=LMAX):
    n = s["npw"]
    fa = flops_per_apply(s, column_shape(s))
    seed_vec = 8.0 * n * (lmax * (lmax + 1) + 6 * lmax + lmax * lmax + 4)
    per_iter = 2 * lmax * fa + seed_vec
    total_iters = float(np.sum(iters))
    gemm = 8.0 * n * (2 * lmax + 2) * (nshift - 1) * total_iters
    return per_iter * total_iters + gemm


def fp64_peak_tflops():
    """Measured FP64 throughput of this GPU: cuBLAS DGEMM 8192^3, best of 5."""
    import torch
    a = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    b = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * 8192 ** 3 / (best * 1e-3) / 1e12


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for k, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(k)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(buf):
    buf.add_(1.0)


def cpu_reference(s, bb, sigma, sample, threads):
    """The reference algorithm (oracle C restatement) on the host cores."""
    from oracle import oracle as O
    O.build()
    op = O.PlaneWaveOperator(s)
    t = time.time()
    x, ierr, iters = O.bicgstab_many(op, bb[:sample], sigma[:sample], lmax=LMAX, threshold=THRESHOLD,
                                     nthreads=threads)
    dt = time.time() - t
    return sample * sigma.shape[1] / dt, dt, iters


def run_reference(args, rank, world):
    if rank != 0:
        return
    s, f, bb, sigma = make_workload()
    threads = os.cpu_count() or 1
    sample = min(bb.shape[0], 32 * threads)
    vals = []  # the CPU path has nothing to warm up; every step is timed
    for k in range(max(1, args.steps)):
        v, dt, iters = cpu_reference(s, bb, sigma, sample, threads)
        vals.append(v)
        log(f"[bench-ref] step {k}: {sample} RHS x {sigma.shape[1]} shifts in {dt:.2f}s -> {v:.1f} solves/s")
    value = float(np.median(vals))
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rhs_per_step": int(bb.shape[0]), "shifts": int(sigma.shape[1])},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} of {bb.shape[0]} right-hand sides x {sigma.shape[1]} shifts per step"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_gpu(args, rank, world):
    import torch
    import torch.distributed as dist

    import sternheimergw_gb300 as sg
    from sternheimergw_gb300 import _capi

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    _capi.lib(build_if_missing=False)
    s, f, bb, sigma = make_workload()
    nrhs, S = sigma.shape
    n = s["npw"]
    op = sg.PlaneWaveOperator(s)
    bb_d = torch.from_numpy(bb).cuda()
    sg_d = torch.from_numpy(sigma).cuda()
    x_d = torch.empty((nrhs, S, n), dtype=torch.complex128, device="cuda")
    l2 = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    precision = 0
    for w in range(args.warmup):
        flush_l2(l2)
        _, ierr, iters = sg.solve_batch(op, bb_d, sg_d, lmax=LMAX, threshold=THRESHOLD, precision=precision, out=x_d)
        ms, _ = op.last_timing()
        log(f"[bench] warmup {w}: {ms:.1f} ms")
    barrier()
    dev_ms, launches, iters_all = [], 0, None
    with ClockSampler(dev) as clk:
        t0 = time.time()
        for k in range(args.steps):
            flush_l2(l2)
            _, ierr, iters = sg.solve_batch(op, bb_d, sg_d, lmax=LMAX, threshold=THRESHOLD, precision=precision,
                                             out=x_d)
            ms, nl = op.last_timing()
            dev_ms.append(ms)
            launches += nl
            iters_all = iters.cpu().numpy()
            log(f"[bench] step {k}: {ms:.1f} ms, ierr max {int(ierr.max())}, iters {iters_all.min()}..{iters_all.max()}")
        barrier()
        wall = time.time() - t0
    ms_step = float(np.mean(dev_ms))
    if world > 1:
        t = torch.tensor([ms_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    solves = nrhs * S
    value = world * solves / (ms_step * 1e-3)

    # end to end through the C ABI with pinned host buffers
    bb_h = torch.from_numpy(bb).pin_memory()
    sg_h = torch.from_numpy(sigma).pin_memory()
    x_h = torch.empty((nrhs, S, n), dtype=torch.complex128).pin_memory()
    e2e_ms = []
    for k in range(max(1, min(args.steps, 2))):
        flush_l2(l2)
        torch.cuda.synchronize()
        t = time.time()
        sg.solve_batch(op, bb_h.numpy(), sg_h.numpy(), lmax=LMAX, threshold=THRESHOLD, precision=precision,
                       out=x_h.numpy())
        e2e_ms.append((time.time() - t) * 1e3)
    e2e_value = world * solves / (float(np.median(e2e_ms)) * 1e-3)
    h2d = bb.nbytes + sigma.nbytes
    d2h = nrhs * S * n * 16 + nrhs * 8

    out = None
    if rank == 0:
        peak = fp64_peak_tflops()
        flops = step_flops(s, iters_all, S)
        achieved = flops / (ms_step * 1e-3) / 1e12
        sample = min(nrhs, 32 * (os.cpu_count() or 1))
        cpu_v, cpu_dt, _ = cpu_reference(s, bb, sigma, sample, os.cpu_count() or 1)
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except OSError:
            pass
        out = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": WORKLOAD, "rhs_per_step": nrhs, "shifts": S, "solves_per_step": solves,
                       "precision": "fp64", "l2": "256 MB buffer written between steps; outputs 4.6 GB > L2",
                       "mean_outer_iterations": float(np.mean(iters_all))},
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": float(np.median(e2e_ms))},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None,
                         "peak_source": "in-run cuBLAS DGEMM 8192^3 (MEASURED_PEAKS.json has no FP64 figure)",
                         "kernel": "msbicg_kernel (one launch per step)", "flops_per_launch": flops},
            "cpu_baseline": {"value": cpu_v, "unit": "solves/s", "cores": os.cpu_count() or 1, "kind": "port",
                             "sample": f"{sample} of {nrhs} right-hand sides x {S} shifts, {cpu_dt:.1f}s"},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "wall_s_timed": wall,
        }
        if peaks.get("hbm_gbs"):
            out["roofline"]["hbm_peak_gbs"] = peaks["hbm_gbs"]
        print(json.dumps(out), flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group(backend)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
