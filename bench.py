"""Benchmark of the batched LU factor-and-solve path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload gesv32]

A step is one batched factor-and-solve of the workload's whole batch.  Each
step works on its own pre-filled copy of the inputs (all copies together are
larger than L2, so no step reads another's data from cache); `value` is
solves/s with inputs resident in HBM, `e2e` is the same metric through the
public C-ABI call with pinned host buffers copied in and the solutions and
info copied out inside the timed region.

--impl reference times the reference's CPU path (LAPACK-style getrf + getrs
per matrix under OpenMP, here the C restatement in oracle/) on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# --------------------------------------------------------------------------
# workloads


def flops_getrf(m, n):
    """testing/flops.h FMULS_GETRF + FADDS_GETRF (real arithmetic)."""
    m, n = float(m), float(n)
    if m < n:
        fmuls = 0.5 * m * (m * (n - m / 3.0 - 1.0) + n) + 2.0 / 3.0 * m
        fadds = 0.5 * m * (m * (n - m / 3.0) - n) + m / 6.0
    else:
        fmuls = 0.5 * n * (n * (m - n / 3.0 - 1.0) + m) + 2.0 / 3.0 * n
        fadds = 0.5 * n * (n * (m - n / 3.0) - m) + n / 6.0
    return fmuls + fadds


def flops_getrs(n, nrhs):
    """testing/flops.h FMULS_GETRS + FADDS_GETRS."""
    n, nrhs = float(n), float(nrhs)
    return nrhs * n * n + nrhs * n * (n - 1.0)


class Gesv32:
    """Plain FP64 magma_dgesv_batched: 10,000 matrices 32x32, one RHS, entries
    uniform(-1,1) from a seeded generator."""
    name = "gesv32"
    batch, n, nrhs = 10000, 32, 1
    dtype = "f64"
    seed = 20240601

    def describe(self):
        return {"workload": "dgesv_batched n=32 nrhs=1 batch=10000 uniform(-1,1) FP64",
                "batch": self.batch, "n": self.n, "nrhs": self.nrhs, "precision": "fp64",
                "matrix": "uniform(-1,1)", "l2": "inputs larger than L2: each step owns its copy"}

    def flops_per_solve(self):
        return flops_getrf(self.n, self.n) + flops_getrs(self.n, self.nrhs)

    def bytes_per_solve(self):
        # A read+write, B read + X write, ipiv, info, three pointers
        n, r = self.n, self.nrhs
        return 16 * n * n + 16 * n * r + 4 * n + 4 + 24

    def host_inputs(self):
        from magma_gb300.testing import colmajor_uniform
        S = colmajor_uniform(self.batch, self.n, self.n, self.n, self.seed)
        X = colmajor_uniform(self.batch, self.nrhs, self.n, self.n, self.seed + 1)
        return S, X


WORKLOADS = {"gesv32": Gesv32}

# --------------------------------------------------------------------------
# helpers


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [l.strip().split(",") for l in self.f.read().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except Exception:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg, dev=None):
    if pg is not None:
        import torch
        if dev is not None:
            pg.barrier(device_ids=[dev.index])
        else:
            pg.barrier()


def allmax(pg, x, dev):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------
# CPU reference leg


def cpu_run(wl, sample, nthreads):
    """Time oracle gesv (C, OpenMP over the batch) on `sample` matrices.  Returns
    seconds for one pass (median of 3) and the thread count."""
    import oracle
    S, X = wl.host_inputs()
    S, X = S[:sample].copy(), X[:sample].copy()
    times = []
    for _ in range(3):
        s, x = S.copy(), X.copy()
        t0 = time.perf_counter()
        oracle.dgesv_batched(s, x, nthreads=nthreads)
        times.append(time.perf_counter() - t0)
    return statistics.median(times), nthreads


def cpu_baseline(wl, target_s=3.0):
    import oracle
    nthreads = oracle.max_threads()
    probe = min(wl.batch, 500)
    t, _ = cpu_run(wl, probe, nthreads)
    sample = int(min(wl.batch, max(probe, probe * target_s / max(t, 1e-6) / 3)))
    t, _ = cpu_run(wl, sample, nthreads)
    return {"value": sample / t, "unit": "solves/s", "cores": nthreads, "kind": "port",
            "sample": f"{sample} of the {wl.batch} matrices of the workload, oracle/lu_oracle.c "
                      f"getrf+getrs per matrix, OpenMP schedule(dynamic) over {nthreads} threads, "
                      f"median of 3 passes"}


def run_reference(args, wl):
    world, rank, local, pg = dist_setup()
    if rank != 0:
        return 0
    import oracle
    nthreads = oracle.max_threads()
    probe = min(wl.batch, 500)
    t, _ = cpu_run(wl, probe, nthreads)
    sample = int(min(wl.batch, max(probe, probe * 2.0 / max(t, 1e-6))))
    S, X = wl.host_inputs()
    S, X = S[:sample].copy(), X[:sample].copy()
    for _ in range(args.warmup):
        oracle.dgesv_batched(S.copy(), X.copy(), nthreads=nthreads)
    times = []
    for _ in range(args.steps):
        s, x = S.copy(), X.copy()
        t0 = time.perf_counter()
        oracle.dgesv_batched(s, x, nthreads=nthreads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = sample * args.steps / tot
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype,
            "data": "synthetic", "config": wl.describe(), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nthreads, "kind": "port",
                             "sample": f"each step: {sample} of the {wl.batch} matrices, "
                                       f"oracle/lu_oracle.c getrf+getrs per matrix, OpenMP over "
                                       f"{nthreads} host threads"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------
# GPU leg

METRIC = "FP64-accurate batched solves/s"


def run_ours(args, wl):
    import torch
    import magma_gb300 as mg
    from magma_gb300 import lib as L
    from magma_gb300.batched import Queue, ptr_array

    world, rank, local, pg = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = L.load()
    stream = torch.cuda.current_stream(dev)
    q = Queue.current(dev)

    S_h, X_h = wl.host_inputs()
    b, n, r = wl.batch, wl.n, wl.nrhs
    nsteps = args.warmup + args.steps
    S0 = torch.from_numpy(S_h).to(dev)
    X0 = torch.from_numpy(X_h).to(dev)
    # one private copy of the inputs per step
    Ss = [S0.clone() for _ in range(nsteps)]
    Xs = [X0.clone() for _ in range(nsteps)]
    ipiv = torch.empty((b, n), dtype=torch.int32, device=dev)
    info = torch.empty((b,), dtype=torch.int32, device=dev)
    dP = ptr_array(ipiv)
    dAs = [ptr_array(s) for s in Ss]
    dBs = [ptr_array(x) for x in Xs]
    fn = lib.magma_dgesv_batched

    def call(i):
        rc = fn(n, r, C.c_void_p(dAs[i].data_ptr()), n, C.c_void_p(dP.data_ptr()),
                C.c_void_p(dBs[i].data_ptr()), n, C.c_void_p(info.data_ptr()), b, q.handle)
        if rc != 0:
            raise RuntimeError(f"magma_dgesv_batched returned {rc}")

    for i in range(args.warmup):
        call(i)
    torch.cuda.synchronize(dev)
    if args.profile:
        # profiling mode: only the timed launches, nothing else (for ncu captures)
        for k in range(args.steps):
            call(args.warmup + k)
        torch.cuda.synchronize(dev)
        return 0

    # peaks for the roofline denominators, measured on this device
    probe = C.CDLL(str(ROOT / "magma_gb300" / "libmlu_probe.so"))
    probe.mlu_probe_fp64_tflops.restype = C.c_double
    probe.mlu_probe_fp64_tflops.argtypes = [C.c_void_p]
    fp64_peak = probe.mlu_probe_fp64_tflops(C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)

    clocks = Clocks(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier(pg, dev)
    torch.cuda.synchronize(dev)
    clocks.start()
    time.sleep(0.3)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        call(args.warmup + k)
        ev[k][1].record(stream)
    end.record(stream)
    torch.cuda.synchronize(dev)
    barrier(pg, dev)
    clk = clocks.stop()
    ms = start.elapsed_time(end)
    ms = allmax(pg, ms, dev)
    per_launch_ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in ev)
    ms_per_step = ms / args.steps
    value = world * b / (ms_per_step * 1e-3)

    # correctness of what was timed: the last step against the accuracy criterion
    A = torch.from_numpy(S_h).to(dev).transpose(1, 2)
    Xsol = Xs[-1][:, :, :n].transpose(1, 2)
    Bm = X0[:, :, :n].transpose(1, 2)
    R = A @ Xsol - Bm
    eps = float(np.finfo(np.float64).eps)
    res = (R.abs().sum(2).amax(1) / (A.abs().sum(2).amax(1) * Xsol.abs().sum(2).amax(1) * n * eps))
    max_res = float(res.max())
    n_ok = int((res <= 30).sum())

    # end to end through the C ABI with pinned host buffers
    hS = torch.from_numpy(S_h).pin_memory()
    hX = torch.from_numpy(X_h).pin_memory()
    hXo = torch.empty_like(hX).pin_memory()
    hInfo = torch.empty((b,), dtype=torch.int32).pin_memory()
    dS, dX = Ss[0], Xs[0]

    def e2e_step():
        dS.copy_(hS, non_blocking=True)
        dX.copy_(hX, non_blocking=True)
        call(0)
        hXo.copy_(dX, non_blocking=True)
        hInfo.copy_(info, non_blocking=True)

    for _ in range(max(args.warmup, 1)):
        e2e_step()
    torch.cuda.synchronize(dev)
    barrier(pg, dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = allmax(pg, e0.elapsed_time(e1), dev) / args.steps
    h2d = hS.numel() * 8 + hX.numel() * 8
    d2h = hXo.numel() * 8 + hInfo.numel() * 4

    if rank != 0:
        return 0
    flops_launch = wl.flops_per_solve() * b
    bytes_launch = wl.bytes_per_solve() * b
    achieved_tf = flops_launch / (per_launch_ms * 1e-3) / 1e12
    cpu = cpu_baseline(wl) if world == 1 else None
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        traffic = json.loads(tfile.read_text()).get(wl.name)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype,
        "data": "synthetic", "config": wl.describe(),
        "roofline": {"bound": "fp64", "achieved": achieved_tf, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": achieved_tf / fp64_peak if fp64_peak > 0 else None,
                     "traffic": traffic,
                     "peak_source": "live FP64 FMA-throughput probe (magma_gb300/probe/peaks.cu)",
                     "kernel": "small_gesv_kernel<double,32,1>",
                     "algorithmic_flops_per_launch": flops_launch,
                     "algorithmic_bytes_per_launch": bytes_launch,
                     "hbm_achieved_gbs": bytes_launch / (per_launch_ms * 1e-3) / 1e9,
                     "hbm_peak_gbs": hbm_peak,
                     "hbm_frac": bytes_launch / (per_launch_ms * 1e-3) / 1e9 / hbm_peak,
                     "launch_ms": per_launch_ms},
        "cpu_baseline": cpu,
        "e2e": {"value": world * b / (e2e_ms * 1e-3), "unit": "solves/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
        "gpu_launches": args.steps,
        "clocks": clk,
        "accuracy": {"max_scaled_residual": max_res, "solves_within_30": n_ok, "of": b},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gesv32", choices=sorted(WORKLOADS))
    ap.add_argument("--profile", action="store_true",
                    help="run warm-up and timed launches only (for ncu), print nothing")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]()
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_ours(args, wl)


if __name__ == "__main__":
    sys.exit(main())
