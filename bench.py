"""Benchmark of the batched LU factor-and-solve path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload dsgesv512|gesv32|vbatched4096|adjoint2048|serve256]
                    [--precision fp32|fp16|bf16] [--solver ir|gmres]
                    [--profile [--batch B] [--eager]]

Metric: FP64-accurate batched solves/s -- solves per second that meet the
reference tester's accuracy bar ||b - A x||_inf / (||A||_inf ||x||_inf n eps)
<= 30 (testing/testing_zgesv_batched.cpp:131-152).

Workloads
  dsgesv512 (default)  512 double matrices n=512, A = U diag(s) V^T with s
                       geometric from 1 to 1/kappa, kappa in {1e2,1e4,1e6} (a
                       third each), nrhs=4 uniform(-1,1).  A step is one call of
                       magma_dsgesv_batched_work (FP32 LU, FP64 residual and
                       update, stop at scaled residual <= 30 or 30 iterations,
                       FP64 re-solve of any matrix that does not converge).  The
                       plain FP64 path (magma_dgesv_batched) is timed on the same
                       inputs and reported beside it.
  gesv32               magma_dgesv_batched on 10,000 matrices 32x32, nrhs=1,
                       uniform(-1,1).

`value` is measured with the inputs resident in HBM (each step reads more
than L2 holds); `e2e` is the same metric through the C-ABI call with pinned
host buffers: inputs copied in and solutions + info copied out inside the
timed region.  --impl reference times the reference's CPU path (LAPACK-style
dgetrf + dgetrs per matrix under OpenMP: the C restatement in oracle/) on the
host cores for the same workload.
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

METRIC = "FP64-accurate batched solves/s"
EPS = float(np.finfo(np.float64).eps)


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


def scaled_residuals(A, X, B):
    """Per-matrix ||B - A X||_inf / (||A||_inf ||X||_inf n eps), torch, math orientation."""
    n = A.shape[1]
    R = A @ X - B
    return R.abs().sum(2).amax(1) / (A.abs().sum(2).amax(1) * X.abs().sum(2).amax(1) * n * EPS)


def vp(t):
    return C.c_void_p(t.data_ptr())


# --------------------------------------------------------------------------
# workloads


class Gesv32:
    name = "gesv32"
    batch, n, nrhs = 10000, 32, 1
    seed = 20240601
    dtype = "f64"

    def describe(self):
        return {"workload": "magma_dgesv_batched n=32 nrhs=1 batch=10000 uniform(-1,1) FP64",
                "batch": self.batch, "n": self.n, "nrhs": self.nrhs, "precision": "fp64",
                "matrix": "uniform(-1,1)",
                "l2": "inputs larger than L2: each step owns a private 85 MB copy"}

    def host_inputs(self):
        from magma_gb300.testing import colmajor_uniform
        S = colmajor_uniform(self.batch, self.n, self.n, self.n, self.seed)
        B = colmajor_uniform(self.batch, self.nrhs, self.n, self.n, self.seed + 1)
        return S, B

    def setup(self, dev, nsteps, lib, q):
        import torch
        from magma_gb300.batched import ptr_array
        S_h, B_h = self.host_inputs()
        c = {"S_h": S_h, "B_h": B_h}
        S0 = torch.from_numpy(S_h).to(dev)
        B0 = torch.from_numpy(B_h).to(dev)
        c["S0"], c["B0"] = S0, B0
        c["S"] = [S0.clone() for _ in range(nsteps)]
        c["X"] = [B0.clone() for _ in range(nsteps)]
        c["dA"] = [ptr_array(s) for s in c["S"]]
        c["dX"] = [ptr_array(x) for x in c["X"]]
        c["ipiv"] = torch.empty((self.batch, self.n), dtype=torch.int32, device=dev)
        c["info"] = torch.empty((self.batch,), dtype=torch.int32, device=dev)
        c["dP"] = ptr_array(c["ipiv"])
        c["lib"], c["q"] = lib, q
        return c

    def step(self, c, i):
        rc = c["lib"].magma_dgesv_batched(self.n, self.nrhs, vp(c["dA"][i]), self.n, vp(c["dP"]),
                                          vp(c["dX"][i]), self.n, vp(c["info"]), self.batch,
                                          c["q"].handle)
        if rc != 0:
            raise RuntimeError(f"magma_dgesv_batched returned {rc}")

    dominant_class = "small_gesv"
    dominant = "mlu::small_gesv_kernel<double,32,1>"

    # End to end: two calls on the two halves of the batch; the second half's host-to-device
    # copy runs on a copy stream while the first half is solved, and each half's solutions
    # go back as soon as it is done.  (Measured on GB300: 0.77 ms per step, 0.84 as one call.)
    E2E_HALVES = 2

    def e2e_setup(self, c):
        import torch
        from magma_gb300.batched import ptr_array
        c["hS"] = torch.from_numpy(c["S_h"]).pin_memory()
        c["hB"] = torch.from_numpy(c["B_h"]).pin_memory()
        c["hX"] = torch.empty_like(c["hB"]).pin_memory()
        c["hInfo"] = torch.empty((self.batch,), dtype=torch.int32).pin_memory()
        c["copy_stream"] = torch.cuda.Stream()
        bounds = np.linspace(0, self.batch, self.E2E_HALVES + 1).astype(int)
        c["halves"] = []
        for k in range(self.E2E_HALVES):
            sl = slice(int(bounds[k]), int(bounds[k + 1]))
            c["halves"].append({"sl": sl, "dA": ptr_array(c["S"][0][sl]), "dX": ptr_array(c["X"][0][sl]),
                                "dP": ptr_array(c["ipiv"][sl])})
        h2d = c["hS"].numel() * 8 + c["hB"].numel() * 8
        d2h = c["hX"].numel() * 8 + c["hInfo"].numel() * 4
        return h2d, d2h

    def e2e_step(self, c):
        import torch
        main, cs = torch.cuda.current_stream(), c["copy_stream"]
        cs.wait_stream(main)                      # the previous step is done with the buffers
        arrived = []
        with torch.cuda.stream(cs):
            for hf in c["halves"]:
                sl = hf["sl"]
                c["S"][0][sl].copy_(c["hS"][sl], non_blocking=True)
                c["X"][0][sl].copy_(c["hB"][sl], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                arrived.append(ev)
        for hf, ev in zip(c["halves"], arrived):
            sl = hf["sl"]
            main.wait_event(ev)
            rc = c["lib"].magma_dgesv_batched(self.n, self.nrhs, vp(hf["dA"]), self.n, vp(hf["dP"]),
                                              vp(hf["dX"]), self.n, vp(c["info"][sl]), sl.stop - sl.start,
                                              c["q"].handle)
            if rc != 0:
                raise RuntimeError(f"magma_dgesv_batched returned {rc}")
            done = torch.cuda.Event()
            done.record(main)
            with torch.cuda.stream(cs):
                cs.wait_event(done)
                c["hX"][sl].copy_(c["X"][0][sl], non_blocking=True)
                c["hInfo"][sl].copy_(c["info"][sl], non_blocking=True)
        main.wait_stream(cs)                      # the step ends when the results are home

    def accuracy(self, c, last):
        n = self.n
        A = c["S0"].transpose(1, 2)
        X = c["X"][last][:, :, :n].transpose(1, 2)
        B = c["B0"][:, :, :n].transpose(1, 2)
        res = scaled_residuals(A, X, B)
        return int((res <= 30).sum()), float(res.max())

    def flops_per_solve(self):
        return flops_getrf(self.n, self.n) + flops_getrs(self.n, self.nrhs)

    def roofline(self, kern, peaks, c):
        flops = self.flops_per_solve() * self.batch          # one launch per step
        n, r = self.n, self.nrhs
        nbytes = (16 * n * n + 16 * n * r + 4 * n + 4 + 24) * self.batch
        ms = kern["launch_ms"]
        ach = flops / (ms * 1e-3) / 1e12
        t = _traffic(self.name)
        return {"bound": "fp64", "achieved": ach, "peak": peaks["fp64_tflops"], "unit": "TFLOP/s",
                "frac": ach / peaks["fp64_tflops"],
                "traffic": None if t is None else t["dram_bytes_per_unit"] * self.batch,
                "traffic_note": None if t is None else t["note"],
                "peak_source": "FP64 FMA-throughput probe run inside bench.py "
                               "(magma_gb300/probe/peaks.cu)",
                **kern, "algorithmic_flops_per_launch": flops,
                "algorithmic_bytes_per_launch": nbytes,
                "hbm_gbs": nbytes / (ms * 1e-3) / 1e9,
                "hbm_frac_of_measured": nbytes / (ms * 1e-3) / 1e9 / peaks["hbm_gbs"]}

    def cpu_sample(self, nthreads, target_s):
        S_h, B_h = self.host_inputs()

        def run(k):
            s, x = S_h[:k].copy(), B_h[:k].copy()
            t0 = time.perf_counter()
            cpu_gesv(s, x, nthreads)
            return time.perf_counter() - t0
        k = min(self.batch, 1000)
        t = run(k)
        k = int(min(self.batch, max(k, k * target_s / max(t, 1e-6))))
        ts = [run(k) for _ in range(3)]
        return k, statistics.median(ts), f"{k} of the {self.batch} matrices"


class Dsgesv512:
    name = "dsgesv512"
    batch, n, nrhs = 512, 512, 4
    seed = 20240603
    dtype = "f64 (FP32 factorisation, FP64 residual/update)"
    tol = 30.0
    itermax = 30
    precision = "fp32"
    solver = "ir"
    SOLVER = {"ir": "FP64 refinement",
              "gmres": "FP64 refinement with each correction solved by FP32 GMRES preconditioned "
                       "with the factors (Magma_REFINE_IRGMSTRS)"}
    FACTOR = {"fp32": "FP32 LU (SIMT FMA)",
              "fp16": "FP32 LU with FP16 tensor-core trailing updates (FP32 accumulation, "
                      "power-of-two row/column scaling)",
              "bf16": "FP32 LU with BF16 tensor-core trailing updates (FP32 accumulation)"}

    def describe(self):
        return {"workload": "magma_dxgesv_batched_work: 512 FP64 matrices n=512, nrhs=4, "
                            "A=U diag(s) V^T, kappa in {1e2,1e4,1e6}; " + self.FACTOR[self.precision]
                            + " + " + self.SOLVER[self.solver]
                            + f", stop at scaled residual <= 30 or {self.itermax} iterations, "
                            "FP64 re-solve of non-converged matrices",
                "batch": self.batch, "n": self.n, "nrhs": self.nrhs,
                "precision": f"{self.precision} factor, fp64 residual/update/convergence",
                "matrix": "svd-type, singular values geometric 1..1/kappa",
                "compared_with": "magma_dgesv_batched (plain FP64) on the same inputs",
                "fp32_getrf_tuning": getattr(self, "tuning", None),
                "autotune_seconds": getattr(self, "tuning_s", None),
                "l2": "inputs larger than L2: A is 1 GiB FP64"}

    def gen(self, dev):
        import torch
        from magma_gb300.testing import svd_batch_torch
        kap = [1e2, 1e4, 1e6] * (self.batch // 3 + 1)
        A = svd_batch_torch(self.batch, self.n, kap[:self.batch], self.seed, device=dev)
        g = torch.Generator(device="cpu").manual_seed(self.seed + 1)
        B = (torch.rand((self.batch, self.n, self.nrhs), generator=g, dtype=torch.float64) * 2
             - 1).to(dev)
        return A, B

    def setup(self, dev, nsteps, lib, q):
        import torch
        import magma_gb300 as mg
        from magma_gb300.batched import ptr_array
        # the fixed-size FP32 factorisation's blocking, timed on this GPU for this order and
        # batch before anything is measured (magma_sgetrf_batched_autotune); --profile runs
        # keep the default table, so that a profiler's launch counts start at the workload
        if not getattr(self, "profile", False):
            t0 = time.perf_counter()
            tuned = mg.autotune_getrf_batched(self.n, self.batch, torch.float32, q)
            self.tuning_s = time.perf_counter() - t0
            self.tuning = {b: v for b, v in tuned.items() if b in ("<=512",)}
        A, B = self.gen(dev)
        c = {"A": A, "Bm": B, "lib": lib, "q": q}
        c["S"] = A.transpose(1, 2).contiguous()          # column-major storage
        c["B"] = B.transpose(1, 2).contiguous()
        c["X"] = torch.empty_like(c["B"])
        b, n = self.batch, self.n
        c["ipiv"] = torch.empty((b, n), dtype=torch.int32, device=dev)
        c["info"] = torch.empty((b,), dtype=torch.int32, device=dev)
        c["iter"] = torch.empty((b,), dtype=torch.int32, device=dev)
        c["work"] = torch.empty((mg.dsgesv_workspace_bytes(n, self.nrhs, b, self.precision,
                                                          self.solver),),
                                dtype=torch.uint8, device=dev)
        c["lwork"] = C.c_size_t(c["work"].numel())
        for k in ("S", "B", "X", "ipiv"):
            c["d" + k] = ptr_array(c[k])
        # a private copy of A per call: a matrix that falls back to the FP64 re-solve has A
        # overwritten by its FP64 factors
        c["Ss"] = [c["S"].clone() for _ in range(nsteps)]
        c["dSs"] = [ptr_array(x) for x in c["Ss"]]
        return c

    def step(self, c, i):
        from magma_gb300.batched import PRECISIONS, SOLVERS
        b, n, r = self.batch, self.n, self.nrhs
        rc = c["lib"].magma_dxgesv_gmres_batched_work(
            PRECISIONS[self.precision], SOLVERS[self.solver], n, r, vp(c["dSs"][i]), n,
            vp(c["dipiv"]), vp(c["dB"]), n, vp(c["dX"]), n, vp(c["info"]), vp(c["iter"]),
            self.itermax, self.tol, 1, vp(c["work"]), C.byref(c["lwork"]), b, c["q"].handle)
        if rc != 0:
            raise RuntimeError(f"magma_dxgesv_gmres_batched_work({self.precision}, {self.solver}) "
                               f"returned {rc}")

    dominant_class = "ir_residual"
    dominant = "mlu::ir_residual_kernel<4> (FP64 residual R = B - A X)"
    # kernel classes timed one at a time in extra calls after the timed region
    breakdown_classes = ("ir_residual", "outer", "ir_solve", "gemm", "panel", "swap_trsm", "ir_init")

    def outer_flops(self):
        """Algorithmic flops of the rank-128 updates (U12 solve + A22 update) of one FP32
        factorisation of order n, two-level blocked (128-column blocks): 2 FMA counts."""
        n, fmas = self.n, 0
        for J in range(0, n, 128):
            K = min(128, n - J)
            E = J + K
            if E < n:
                fmas += K * (K - 1) // 2 * (n - E) + (n - E) * (n - E) * K
        return 2.0 * fmas

    def restore(self, c, i):
        """A private copy back to the input (a matrix that fell back to FP64 has its A
        overwritten by FP64 factors)."""
        c["Ss"][i].copy_(c["S"])

    def secondary_roofline(self, times, peaks):
        """The rank-128 update kernel (FP32 SIMT FMA): its algorithmic flops per step over
        its measured time per step, against the FP32 FMA rate probed in the same run."""
        if "outer" not in times or times["outer"] <= 0:
            return None
        flops = self.outer_flops() * self.batch
        ach = flops / (times["outer"] * 1e-3) / 1e12
        return {"kernel": "mlu::outer_update_kernel (FP32 interchanges + U12 solve + rank-128 "
                          "A22 update)", "bound": "fp32", "achieved": ach,
                "peak": peaks["fp32_tflops"], "unit": "TFLOP/s", "frac": ach / peaks["fp32_tflops"],
                "algorithmic_flops_per_step": flops, "ms_per_step": times["outer"],
                "peak_source": "FP32 FMA-throughput probe run inside bench.py "
                               "(magma_gb300/probe/peaks.cu)"}

    # End to end: the batch goes through the C ABI as several calls on consecutive slices
    # (E2E_SPLITS, fractions of the batch), issued round-robin on E2E_STREAMS queues (each
    # with its own workspace); all host-to-device copies are queued at once on a copy
    # stream, so later slices arrive while earlier ones are solved, and each slice's
    # solutions go back as soon as it is done.  Measured on GB300 (ms per step of 512
    # matrices): two halves on two queues 11.4; quarters on two queues 12.5; a quarter then
    # three quarters on one queue 11.7-18.5 (the host's wake-up after each call's final
    # read stays on the critical path with one queue, so it follows the host's load).
    E2E_SPLITS = (0.5, 0.5)
    E2E_STREAMS = 2

    def e2e_setup(self, c):
        import torch
        import magma_gb300 as mg
        from magma_gb300.batched import ptr_array, Queue
        c["hS"] = c["S"].cpu().pin_memory()
        c["hB"] = c["B"].cpu().pin_memory()
        c["hX"] = torch.empty_like(c["hB"]).pin_memory()
        c["hIter"] = torch.empty((self.batch,), dtype=torch.int32).pin_memory()
        c["hInfo"] = torch.empty((self.batch,), dtype=torch.int32).pin_memory()
        c["copy_stream"] = torch.cuda.Stream()
        dev = c["S"].device
        c["e2e_q"] = [(torch.cuda.current_stream(), c["q"], c["work"], c["lwork"])]
        for _ in range(1, self.E2E_STREAMS):
            st = torch.cuda.Stream()
            w = torch.empty_like(c["work"])
            c["e2e_q"].append((st, Queue(dev.index, st.cuda_stream), w, C.c_size_t(w.numel())))
        bounds = np.round(np.cumsum((0.0,) + tuple(self.E2E_SPLITS)) * self.batch).astype(int)
        c["chunks"] = []
        for k in range(len(self.E2E_SPLITS)):
            sl = slice(int(bounds[k]), int(bounds[k + 1]))
            c["chunks"].append({"sl": sl, "dS": ptr_array(c["Ss"][0][sl]), "dB": ptr_array(c["B"][sl]),
                                "dX": ptr_array(c["X"][sl]), "dP": ptr_array(c["ipiv"][sl]),
                                "qi": k % self.E2E_STREAMS})
        h2d = c["hS"].numel() * 8 + c["hB"].numel() * 8
        d2h = c["hX"].numel() * 8 + 8 * self.batch
        return h2d, d2h

    def e2e_step(self, c):
        import torch
        from magma_gb300.batched import PRECISIONS, SOLVERS
        main, cs = torch.cuda.current_stream(), c["copy_stream"]
        cs.wait_stream(main)                      # the previous step is done with the buffers
        arrived = []
        with torch.cuda.stream(cs):
            for ck in c["chunks"]:
                sl = ck["sl"]
                c["Ss"][0][sl].copy_(c["hS"][sl], non_blocking=True)
                c["B"][sl].copy_(c["hB"][sl], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                arrived.append(ev)
        n, r = self.n, self.nrhs

        def run(qi):
            # the calls of one queue, in order; a call returns once its slice is solved (it
            # reads the count of matrices that need the FP64 re-solve), so several queues
            # are driven from separate host threads
            for ck, ev in zip(c["chunks"], arrived):
                if ck["qi"] != qi:
                    continue
                sl = ck["sl"]
                st, q, work, lwork = c["e2e_q"][qi]
                st.wait_event(ev)
                rc = c["lib"].magma_dxgesv_gmres_batched_work(
                    PRECISIONS[self.precision], SOLVERS[self.solver], n, r, vp(ck["dS"]), n,
                    vp(ck["dP"]), vp(ck["dB"]), n, vp(ck["dX"]), n, vp(c["info"][sl]),
                    vp(c["iter"][sl]), self.itermax, self.tol, 1, vp(work), C.byref(lwork),
                    sl.stop - sl.start, q.handle)
                if rc != 0:
                    raise RuntimeError(f"magma_dxgesv_gmres_batched_work returned {rc}")
                done = torch.cuda.Event()
                done.record(st)
                with torch.cuda.stream(cs):
                    cs.wait_event(done)
                    c["hX"][sl].copy_(c["X"][sl], non_blocking=True)
                    c["hIter"][sl].copy_(c["iter"][sl], non_blocking=True)
                    c["hInfo"][sl].copy_(c["info"][sl], non_blocking=True)
        if self.E2E_STREAMS == 1:
            run(0)
        else:
            if "pool" not in c:
                import concurrent.futures as cf
                c["pool"] = cf.ThreadPoolExecutor(self.E2E_STREAMS)
            for f in [c["pool"].submit(run, qi) for qi in range(self.E2E_STREAMS)]:
                f.result()
        for st, _, _, _ in c["e2e_q"]:
            main.wait_stream(st)
        main.wait_stream(cs)                      # the step ends when the results are home

    def accuracy(self, c, last):
        X = c["X"].transpose(1, 2)
        res = scaled_residuals(c["A"], X, c["Bm"])
        it = c["iter"].cpu().numpy()
        kap = np.array(([1e2, 1e4, 1e6] * (self.batch // 3 + 1))[:self.batch])
        per = {}
        for kv in (1e2, 1e4, 1e6):
            sel = it[kap == kv]
            per[f"{kv:.0e}"] = {"iterations_histogram": {str(int(k)): int(v) for k, v in
                                                          zip(*np.unique(sel, return_counts=True))},
                                "fallbacks": int((sel < 0).sum())}
        return int((res <= 30).sum()), float(res.max()), {
            "iterations_histogram": {str(int(k)): int(v) for k, v in
                                     zip(*np.unique(it, return_counts=True))},
            "fallbacks": int((it < 0).sum()), "by_kappa": per}

    def fp64_path(self, c, steps, warmup):
        """Plain FP64 magma_dgesv_batched on the same inputs, private copies per step."""
        import torch
        from magma_gb300.batched import ptr_array
        b, n, r = self.batch, self.n, self.nrhs
        stream = torch.cuda.current_stream()
        tot = steps + warmup
        Ss = [c["S"].clone() for _ in range(tot)]
        Xs = [c["B"].clone() for _ in range(tot)]
        dS = [ptr_array(s) for s in Ss]
        dX = [ptr_array(x) for x in Xs]
        lib, q = c["lib"], c["q"]

        def call(i):
            rc = lib.magma_dgesv_batched(n, r, vp(dS[i]), n, vp(c["dipiv"]), vp(dX[i]), n,
                                         vp(c["info"]), b, q.handle)
            if rc != 0:
                raise RuntimeError(f"magma_dgesv_batched returned {rc}")
        for i in range(warmup):
            call(i)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(steps):
            call(warmup + i)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        res = scaled_residuals(c["A"], Xs[-1].transpose(1, 2), c["Bm"])
        n_ok = int((res <= 30).sum())
        del Ss, Xs
        return {"value": n_ok / (ms * 1e-3), "unit": "solves/s", "ms_per_step": ms,
                "max_scaled_residual": float(res.max()), "steps": steps,
                "call": "magma_dgesv_batched"}

    def passes(self, c):
        """Residual passes per matrix in the last step: the initial residual plus one per
        iteration (itermax + 1 for a matrix that did not converge)."""
        it = c["iter"].cpu().numpy()
        return np.where(it >= 0, it + 1, self.itermax + 1)

    def roofline(self, kern, peaks, c):
        n, r, b = self.n, self.nrhs, self.batch
        ms_step = kern["ms"] / kern["steps"]
        if self.dominant_class == "ir_residual":
            # 2 n^2 r FP64 flops per matrix and pass; A read once per pass (FP64)
            passes = int(self.passes(c).sum())
            flops = 2.0 * n * n * r * passes
            nbytes = (8.0 * n * n + 3 * 8.0 * n * r) * passes
            peak, unit, bound = peaks["fp64_tflops"], "TFLOP/s", "fp64"
            src = "FP64 FMA-throughput probe run inside bench.py (magma_gb300/probe/peaks.cu)"
            ach = flops / (ms_step * 1e-3) / 1e12
            extra = {"residual_passes_per_step": passes}
        else:
            raise ValueError(self.dominant_class)
        t = _traffic(self.name)
        traffic = None if t is None else t["dram_bytes_per_unit"] * passes
        return {"bound": bound, "achieved": ach, "peak": peak, "unit": unit, "frac": ach / peak,
                "traffic": traffic, "traffic_note": None if t is None else t["note"],
                "peak_source": src, **kern,
                "algorithmic_flops_per_step": flops, "algorithmic_bytes_per_step": nbytes,
                "hbm_gbs": nbytes / (ms_step * 1e-3) / 1e9,
                "hbm_frac_of_measured": nbytes / (ms_step * 1e-3) / 1e9 / peaks["hbm_gbs"],
                **extra}

    def cpu_sample(self, nthreads, target_s):
        if not hasattr(self, "_cpu_inputs"):
            A, B = self.gen("cpu")
            self._cpu_inputs = (A.transpose(1, 2).contiguous().numpy(),
                                B.transpose(1, 2).contiguous().numpy())
        S, Bs = self._cpu_inputs

        def run(k):
            s, x = S[:k].copy(), Bs[:k].copy()
            t0 = time.perf_counter()
            cpu_gesv(s, x, nthreads)
            return time.perf_counter() - t0
        k = max(nthreads, 1)
        t = run(k)
        k = int(min(self.batch, max(k, k * target_s / max(t, 1e-6))))
        ts = [run(k) for _ in range(3)]
        return k, statistics.median(ts), f"{k} of the {self.batch} matrices (FP64 dgesv)"


class GesvVbatched:
    """Variable-size FP64 factor+solve (magma_dgesv_vbatched_max_nocheck_work,
    one persistent launch after a device-side size sort), CUDA-graph captured."""
    name = "vbatched4096"
    batch = 4096
    seed = 20240602
    dtype = "f64"

    def describe(self):
        return {"workload": "magma_dgesv_vbatched: 4096 FP64 matrices, n uniform in [8,256], "
                            "nrhs uniform in [1,16], entries uniform(-1,1); one persistent "
                            "size-sorted launch replayed from a CUDA graph",
                "batch": self.batch, "n": "U[8,256]", "nrhs": "U[1,16]", "precision": "fp64",
                "autotuned": {b: v for b, v in getattr(self, "tuning", {}).items()
                              if b in ("<=16", "<=32", "<=64", "<=128", "<=256")},
                "autotune_seconds": getattr(self, "tuning_s", None),
                "l2": "inputs larger than L2: each step owns a private copy (~0.7 GB)"}

    def sizes(self):
        rng = np.random.default_rng(self.seed)
        ns = rng.integers(8, 257, self.batch)
        rs = rng.integers(1, 17, self.batch)
        return [int(x) for x in ns], [int(x) for x in rs]

    def host_inputs(self):
        ns, rs = self.sizes()
        rng = np.random.default_rng(self.seed + 1)
        As = [rng.uniform(-1, 1, (n, n)) for n in ns]     # storage (ncols, ld)
        Bs = [rng.uniform(-1, 1, (r, n)) for n, r in zip(ns, rs)]
        return ns, rs, As, Bs

    def flops_total(self):
        ns, rs = self.sizes()
        return sum(flops_getrf(n, n) + flops_getrs(n, r) for n, r in zip(ns, rs))

    def setup(self, dev, nsteps, lib, q):
        import torch
        from magma_gb300.batched import VBatch, Queue
        import magma_gb300 as mg
        ns, rs, As, Bs = self.host_inputs()
        c = {"ns": ns, "rs": rs, "As": As, "Bs": Bs, "lib": lib}
        # panel width and update tile per size bin, timed on this GPU before the graphs are
        # captured (the captured launches read the installed table)
        t0 = time.perf_counter()
        self.tuning = mg.autotune_vbatched(max(ns), torch.float64, q)
        self.tuning_s = time.perf_counter() - t0
        A0 = VBatch([a.shape for a in As], ns, torch.float64, dev).load(As)
        B0 = VBatch([b.shape for b in Bs], ns, torch.float64, dev).load(Bs)
        c["A0"], c["B0"] = A0, B0
        offs = np.concatenate([[0], np.cumsum(ns)[:-1]])
        c["ipiv"] = torch.zeros((sum(ns),), dtype=torch.int32, device=dev)
        c["dP"] = c["ipiv"].data_ptr() + torch.tensor(offs, dtype=torch.int64, device=dev) * 4
        c["info"] = torch.empty((self.batch,), dtype=torch.int32, device=dev)
        lw = C.c_int(-1)
        lib.magma_dgesv_vbatched_max_nocheck_work(None, None, 256, 16, None, None, None, None,
                                                  None, None, None, C.byref(lw), self.batch, None)
        c["lwork"] = lw
        c["work"] = torch.empty((lw.value,), dtype=torch.uint8, device=dev)
        # one private copy per step, each with its own captured graph
        c["A"], c["B"], c["graphs"] = [], [], []
        stream = torch.cuda.Stream(dev)
        c["gstream"] = stream
        c["gq"] = Queue(dev.index, stream.cuda_stream)
        for i in range(nsteps):
            A = VBatch(A0.shapes, ns, torch.float64, dev)
            B = VBatch(B0.shapes, ns, torch.float64, dev)
            A.buf.copy_(A0.buf)
            B.buf.copy_(B0.buf)
            c["A"].append(A)
            c["B"].append(B)
        torch.cuda.synchronize(dev)
        for i in range(nsteps):
            A, B = c["A"][i], c["B"][i]
            with torch.cuda.stream(stream):
                self._call(c, A, B, c["gq"])          # eager once (kernel attributes)
                stream.synchronize()
                A.buf.copy_(A0.buf)
                B.buf.copy_(B0.buf)
                stream.synchronize()
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g, stream=stream):
                    self._call(c, A, B, c["gq"])
            c["graphs"].append(g)
        torch.cuda.synchronize(dev)
        return c

    def _call(self, c, A, B, q):
        rc = c["lib"].magma_dgesv_vbatched_max_nocheck_work(
            vp(A.ncols), vp(B.ncols), 256, 16, vp(A.ptrs), vp(A.ld), vp(c["dP"]), vp(B.ptrs),
            vp(B.ld), vp(c["info"]), vp(c["work"]), C.byref(c["lwork"]), c.get("b", self.batch),
            q.handle)
        if rc != 0:
            raise RuntimeError(f"magma_dgesv_vbatched_max_nocheck_work returned {rc}")

    def step(self, c, i):
        if getattr(self, "eager", False):         # --profile --eager: the same call, no graph
            self._call(c, c["A"][i], c["B"][i], c["gq"])
        else:
            c["graphs"][i].replay()

    dominant_class = None        # graph replay: the step is the sort + the persistent kernel
    graph_kernels_per_step = 2
    dominant = "mlu::vb_lu_kernel<double> (persistent)"

    # End to end: the batch as two halves, each with its own buffers and captured graph; the
    # second half's inputs arrive on a copy stream while the first half's graph runs, and each
    # half's solutions go back as soon as its graph is done.  (Measured on GB300: 26.2 ms per
    # step, 31.7 as one graph.)
    E2E_HALVES = 2

    def _half(self, dev, lib, ns, As, Bs):
        """Buffers, workspace and a captured graph for the matrices given."""
        import torch
        from magma_gb300.batched import VBatch, Queue
        b = len(ns)
        hc = {"lib": lib, "b": b}
        hc["A"] = VBatch([a.shape for a in As], ns, torch.float64, dev).load(As)
        hc["B"] = VBatch([x.shape for x in Bs], ns, torch.float64, dev).load(Bs)
        offs = np.concatenate([[0], np.cumsum(ns)[:-1]])
        hc["ipiv"] = torch.zeros((sum(ns),), dtype=torch.int32, device=dev)
        hc["dP"] = hc["ipiv"].data_ptr() + torch.tensor(offs, dtype=torch.int64, device=dev) * 4
        hc["info"] = torch.empty((b,), dtype=torch.int32, device=dev)
        lw = C.c_int(-1)
        lib.magma_dgesv_vbatched_max_nocheck_work(None, None, 256, 16, None, None, None, None,
                                                  None, None, None, C.byref(lw), b, None)
        hc["lwork"] = lw
        hc["work"] = torch.empty((lw.value,), dtype=torch.uint8, device=dev)
        stream = torch.cuda.Stream(dev)
        hc["gq"] = Queue(dev.index, stream.cuda_stream)
        torch.cuda.synchronize(dev)
        with torch.cuda.stream(stream):
            self._call(hc, hc["A"], hc["B"], hc["gq"])   # eager once (kernel attributes)
            stream.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                self._call(hc, hc["A"], hc["B"], hc["gq"])
        hc["graph"] = g
        hc["hA"] = hc["A"].buf.cpu().pin_memory()
        hc["hB"] = hc["B"].buf.cpu().pin_memory()
        hc["hX"] = torch.empty_like(hc["hB"]).pin_memory()
        hc["hInfo"] = torch.empty((b,), dtype=torch.int32).pin_memory()
        torch.cuda.synchronize(dev)
        return hc

    def e2e_setup(self, c):
        import torch
        dev = c["A0"].buf.device
        ns, As, Bs = c["ns"], c["As"], c["Bs"]
        h = len(ns) // 2
        c["e2e_halves"] = [self._half(dev, c["lib"], ns[lo:hi], As[lo:hi], Bs[lo:hi])
                           for lo, hi in ((0, h), (h, len(ns)))]
        c["copy_stream"] = torch.cuda.Stream(dev)
        h2d = sum(hc["hA"].numel() * 8 + hc["hB"].numel() * 8 for hc in c["e2e_halves"])
        d2h = sum(hc["hX"].numel() * 8 + hc["b"] * 4 for hc in c["e2e_halves"])
        return h2d, d2h

    def e2e_step(self, c):
        import torch
        main, cs = torch.cuda.current_stream(), c["copy_stream"]
        cs.wait_stream(main)                      # the previous step is done with the buffers
        arrived = []
        with torch.cuda.stream(cs):
            for hc in c["e2e_halves"]:
                hc["A"].buf.copy_(hc["hA"], non_blocking=True)
                hc["B"].buf.copy_(hc["hB"], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                arrived.append(ev)
        for hc, ev in zip(c["e2e_halves"], arrived):
            main.wait_event(ev)
            hc["graph"].replay()
            done = torch.cuda.Event()
            done.record(main)
            with torch.cuda.stream(cs):
                cs.wait_event(done)
                hc["hX"].copy_(hc["B"].buf, non_blocking=True)
                hc["hInfo"].copy_(hc["info"], non_blocking=True)
        main.wait_stream(cs)                      # the step ends when the results are home

    def accuracy(self, c, last):
        import torch
        ns, rs, As, Bs = c["ns"], c["rs"], c["As"], c["Bs"]
        B = c["B"][last]
        worst, ok = 0.0, 0
        for k in range(self.batch):
            A = torch.from_numpy(As[k].T.copy())
            X = B.view(k).cpu().T
            Bm = torch.from_numpy(Bs[k].T.copy())
            r = float(scaled_residuals(A[None], X[None], Bm[None])[0])
            worst = max(worst, r)
            ok += r <= 30
        return ok, worst

    def roofline(self, kern, peaks, c):
        flops = self.flops_total()
        ms = kern["launch_ms"]
        ach = flops / (ms * 1e-3) / 1e12
        return {"bound": "fp64", "achieved": ach, "peak": peaks["fp64_tflops"], "unit": "TFLOP/s",
                "frac": ach / peaks["fp64_tflops"], "traffic": _traffic(self.name),
                "peak_source": "FP64 FMA-throughput probe run inside bench.py",
                **kern, "algorithmic_flops_per_launch": flops,
                "note": "timed as the CUDA-graph replay (size sort + persistent kernel); the "
                        "sort's share of the replay is in the launch-list summary"}

    def cpu_sample(self, nthreads, target_s):
        ns, rs, As, Bs = self.host_inputs()

        def run(k):
            a = [x.copy() for x in As[:k]]
            b = [x.copy() for x in Bs[:k]]
            t0 = time.perf_counter()
            cpu_gesv_list(ns[:k], rs[:k], a, b, nthreads)
            return time.perf_counter() - t0
        k = 256
        t = run(k)
        k = int(min(self.batch, max(k, k * target_s / max(t, 1e-6))))
        ts = [run(k) for _ in range(3)]
        return k, statistics.median(ts), f"the first {k} of the {self.batch} matrices"


class Adjoint2048:
    """Differentiable solve: forward magma_dgesv_batched + backward
    magma_dgesv_adjoint_batched through magma_gb300.autograd.solve."""
    name = "adjoint2048"
    batch, n, nrhs = 2048, 64, 4
    seed = 20240604
    dtype = "f64"

    def describe(self):
        return {"workload": "autograd solve x = A^{-1} b, forward + backward: 2048 FP64 matrices "
                            "n=64, A = 4I + uniform(-1,1), nrhs=4, upstream gradient N(0,1)",
                "batch": self.batch, "n": self.n, "nrhs": self.nrhs, "precision": "fp64",
                "l2": "each step owns its inputs (34 MB) and writes gA (34 MB)"}

    def setup(self, dev, nsteps, lib, q):
        import torch
        g = torch.Generator(device="cpu").manual_seed(self.seed)
        b, n, r = self.batch, self.n, self.nrhs
        A = 4.0 * torch.eye(n, dtype=torch.float64) + (torch.rand((b, n, n), generator=g,
                                                                  dtype=torch.float64) * 2 - 1)
        B = torch.rand((b, n, r), generator=g, dtype=torch.float64) * 2 - 1
        gX = torch.randn((b, n, r), generator=g, dtype=torch.float64)
        c = {"A0": A.to(dev), "B0": B.to(dev), "gX": gX.to(dev)}
        c["hA"], c["hB"], c["hgX"] = A.pin_memory(), B.pin_memory(), gX.pin_memory()
        c["As"] = [c["A0"].clone().requires_grad_(True) for _ in range(nsteps)]
        c["Bs"] = [c["B0"].clone().requires_grad_(True) for _ in range(nsteps)]
        return c

    def step(self, c, i):
        from magma_gb300.autograd import solve
        A, B = c["As"][i], c["Bs"][i]
        A.grad = None
        B.grad = None
        X = solve(A, B)
        X.backward(c["gX"])
        c["last_X"] = X

    dominant_class = "getrs"
    dominant = "triangular solves (forward getrs and transposed adjoint getrs)"

    def e2e_setup(self, c):
        import torch
        c["hgA"] = torch.empty((self.batch, self.n, self.n), dtype=torch.float64).pin_memory()
        c["hgB"] = torch.empty((self.batch, self.n, self.nrhs), dtype=torch.float64).pin_memory()
        c["dA"] = torch.empty_like(c["A0"])
        c["dB"] = torch.empty_like(c["B0"])
        c["dg"] = torch.empty_like(c["gX"])
        c["copy_stream"] = torch.cuda.Stream()
        h2d = (c["hA"].numel() + c["hB"].numel() + c["hgX"].numel()) * 8
        d2h = (c["hgA"].numel() + c["hgB"].numel()) * 8
        return h2d, d2h

    # End to end: the batch as two halves, each its own forward + backward; the second half's
    # inputs arrive on a copy stream while the first is solved, and each half's gradients go
    # back as soon as they are computed.  (Measured on GB300: 1.88 ms per step, 1.96 as one pass.)
    E2E_HALVES = 2

    def e2e_step(self, c):
        import torch
        from magma_gb300.autograd import solve
        main, cs = torch.cuda.current_stream(), c["copy_stream"]
        cs.wait_stream(main)                      # the previous step is done with the buffers
        bounds = np.linspace(0, self.batch, self.E2E_HALVES + 1).astype(int)
        halves = [slice(int(bounds[k]), int(bounds[k + 1])) for k in range(self.E2E_HALVES)]
        arrived = []
        with torch.cuda.stream(cs):
            for sl in halves:
                c["dA"][sl].copy_(c["hA"][sl], non_blocking=True)
                c["dB"][sl].copy_(c["hB"][sl], non_blocking=True)
                c["dg"][sl].copy_(c["hgX"][sl], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                arrived.append(ev)
        for sl, ev in zip(halves, arrived):
            main.wait_event(ev)
            A = c["dA"][sl].detach().requires_grad_(True)
            B = c["dB"][sl].detach().requires_grad_(True)
            solve(A, B).backward(c["dg"][sl])
            done = torch.cuda.Event()
            done.record(main)
            gA, gB = A.grad, B.grad
            with torch.cuda.stream(cs):
                cs.wait_event(done)
                c["hgA"][sl].copy_(gA, non_blocking=True)
                c["hgB"][sl].copy_(gB, non_blocking=True)
                gA.record_stream(cs)
                gB.record_stream(cs)
        main.wait_stream(cs)                      # the step ends when the gradients are home

    def accuracy(self, c, last):
        import torch
        A = c["A0"].clone().requires_grad_(True)
        B = c["B0"].clone().requires_grad_(True)
        X = torch.linalg.solve(A, B)
        X.backward(c["gX"])
        Ag = c["As"][last].grad
        rel = float((Ag - A.grad).abs().max() / A.grad.abs().max())
        res = scaled_residuals(c["A0"], c["last_X"].detach(), c["B0"])
        return int((res <= 30).sum()), float(res.max()), {"grad_rel_err_vs_torch_fp64": rel}

    def roofline(self, kern, peaks, c):
        # two triangular-solve launches per step (forward solve, transposed solve)
        b, n, r = self.batch, self.n, self.nrhs
        flops = b * 2 * flops_getrs(n, r)
        nbytes = b * 2 * (8.0 * n * n + 2 * 8.0 * n * r + 4 * n)
        ms_step = kern["ms"] / kern["steps"]
        ach = nbytes / (ms_step * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": ach / peaks["hbm_gbs"], "traffic": _traffic(self.name),
                "peak_source": peaks["hbm_source"], **kern,
                "algorithmic_bytes_per_step": nbytes, "algorithmic_flops_per_step": flops,
                "fp64_tflops": flops / (ms_step * 1e-3) / 1e12}

    def cpu_sample(self, nthreads, target_s):
        import torch
        g = torch.Generator(device="cpu").manual_seed(self.seed)
        b, n, r = self.batch, self.n, self.nrhs
        A = 4.0 * torch.eye(n, dtype=torch.float64) + (torch.rand((b, n, n), generator=g,
                                                                  dtype=torch.float64) * 2 - 1)
        B = torch.rand((b, n, r), generator=g, dtype=torch.float64) * 2 - 1
        gX = torch.randn((b, n, r), generator=g, dtype=torch.float64)
        S0 = A.transpose(1, 2).contiguous().numpy()
        X0 = B.transpose(1, 2).contiguous().numpy()
        G0 = gX.transpose(1, 2).contiguous().numpy()

        def run(k):
            S, X, G = S0[:k].copy(), X0[:k].copy(), G0[:k].copy()
            t0 = time.perf_counter()
            cpu_adjoint_list([n] * k, [r] * k, list(S), list(X), list(G), nthreads)
            return time.perf_counter() - t0
        k = 256
        t = run(k)
        k = int(min(b, max(k, k * target_s / max(t, 1e-6))))
        ts = [run(k) for _ in range(3)]
        return k, statistics.median(ts), f"{k} of the {b} forward+backward solves"


class Serve256:
    """Serving-size workload: variable-size refinement solve plus its adjoint, one CUDA graph
    per step (magma_dxgesv_vbatched_work + magma_dxgesv_adjoint_vbatched_work, both without
    host synchronisation), against the plain FP64 variable-size path on the same inputs."""
    name = "serve256"
    batch, nrhs = 256, 8
    seed = 20240605
    dtype = "f64 (FP32 factorisation, FP64 residual/update; FP64-refined adjoint)"
    itermax = 30
    tol = 30.0
    dominant_class = None        # graph replay; see roofline()
    dominant = "one CUDA-graph replay: refinement forward + adjoint"
    graph_kernels_per_step = None

    def describe(self):
        return {"workload": "256 FP64 matrices, n uniform in [128,1024], A = U diag(s) V^T (U, V "
                            "from QR of seeded Gaussians, s geometric 1..1/kappa, kappa "
                            "log-uniform in [1,1e4]), nrhs=8 N(0,1), upstream gradient N(0,1); "
                            "forward: FP32 LU with per-matrix sizes (the per-step two-level "
                            "kernels: orders above the persistent kernel's 256) + FP64 "
                            "refinement; backward: gB = A^-T gX refined in FP64 with the same FP32 "
                            "factors, gA = -gB X^T; one CUDA graph per step",
                "batch": self.batch, "n": "U[128,1024]", "nrhs": self.nrhs,
                "precision": "fp32 factor, fp64 residual/update/convergence, forward and adjoint",
                "compared_with": "magma_dgesv_vbatched + magma_dgetrs_vbatched(MagmaTrans) + "
                                 "magmablas_dger_neg_vbatched (plain FP64) on the same inputs",
                "tensor_core_factor": "not used: BF16/FP16 factors do not converge under plain "
                                      "refinement for kappa up to 1e4 (kappa * u > 1)",
                "l2": "inputs larger than L2 (A is ~0.8 GB FP64)"}

    def sizes(self):
        rng = np.random.default_rng(self.seed)
        ns = [int(x) for x in rng.integers(128, 1025, self.batch)]
        kap = [float(x) for x in 10.0 ** rng.uniform(0.0, 4.0, self.batch)]
        return ns, kap

    def host_inputs(self):
        ns, kap = self.sizes()
        As, Bs, Gs = [], [], []
        for k, (n, kp) in enumerate(zip(ns, kap)):
            rng = np.random.default_rng(self.seed * 7919 + k)
            U = np.linalg.qr(rng.standard_normal((n, n)))[0]
            V = np.linalg.qr(rng.standard_normal((n, n)))[0]
            sv = np.geomspace(1.0, 1.0 / kp, n)
            As.append(np.ascontiguousarray(((U * sv) @ V.T).T))       # storage (ncols, ld=n)
            Bs.append(rng.standard_normal((self.nrhs, n)))
            Gs.append(rng.standard_normal((self.nrhs, n)))
        return ns, As, Bs, Gs

    def flops(self):
        ns, _ = self.sizes()
        return sum(flops_getrf(n, n) for n in ns)

    def _calls(self, c, q):
        lib, b = c["lib"], c["b"]
        A, B, X, G, GB, GA = c["A"], c["B"], c["X"], c["G"], c["GB"], c["GA"]
        rc = lib.magma_dxgesv_vbatched_work(
            900, vp(A.ncols), vp(B.ncols), c["max_n"], self.nrhs, vp(A.ptrs), vp(A.ld),
            vp(c["dP"]), vp(B.ptrs), vp(B.ld), vp(X.ptrs), vp(X.ld), vp(c["info"]),
            vp(c["iter"]), self.itermax, self.tol, 0, vp(c["work"]), C.byref(c["lwork"]), b,
            q.handle)
        if rc != 0:
            raise RuntimeError(f"magma_dxgesv_vbatched_work returned {rc}")
        rc = lib.magma_dxgesv_adjoint_vbatched_work(
            vp(A.ncols), vp(G.ncols), c["max_n"], self.nrhs, vp(A.ptrs), vp(A.ld), vp(c["dP"]),
            vp(X.ptrs), vp(X.ld), vp(G.ptrs), vp(G.ld), vp(GB.ptrs), vp(GB.ld), vp(GA.ptrs),
            vp(GA.ld), vp(c["iter"]), vp(c["info"]), vp(c["iter_adj"]), self.itermax, self.tol, 0,
            vp(c["work"]), c["lwork"].value, b, q.handle)
        if rc != 0:
            raise RuntimeError(f"magma_dxgesv_adjoint_vbatched_work returned {rc}")

    def setup(self, dev, nsteps, lib, q):
        ns, As, Bs, Gs = self.host_inputs()
        return self._context(dev, lib, ns, As, Bs, Gs)

    def _context(self, dev, lib, ns, As, Bs, Gs):
        """Device buffers, workspace and the captured graph for the matrices given."""
        import torch
        from magma_gb300.batched import VBatch, Queue
        c = {"ns": ns, "As": As, "Bs": Bs, "Gs": Gs, "lib": lib, "max_n": max(ns), "b": len(ns)}
        c["A"] = VBatch([a.shape for a in As], ns, torch.float64, dev).load(As)
        c["B"] = VBatch([b.shape for b in Bs], ns, torch.float64, dev).load(Bs)
        c["G"] = VBatch([g.shape for g in Gs], ns, torch.float64, dev).load(Gs)
        c["X"] = VBatch(c["B"].shapes, ns, torch.float64, dev)
        c["GB"] = VBatch(c["G"].shapes, ns, torch.float64, dev)
        c["GA"] = VBatch([(n, n) for n in ns], ns, torch.float64, dev)
        offs = np.concatenate([[0], np.cumsum(ns)[:-1]])
        c["ipiv"] = torch.zeros((sum(ns),), dtype=torch.int32, device=dev)
        c["dP"] = c["ipiv"].data_ptr() + torch.tensor(offs, dtype=torch.int64, device=dev) * 4
        b = len(ns)
        c["info"] = torch.empty((b,), dtype=torch.int32, device=dev)
        c["iter"] = torch.empty((b,), dtype=torch.int32, device=dev)
        c["iter_adj"] = torch.empty((b,), dtype=torch.int32, device=dev)
        lw = C.c_size_t(0)
        rc = lib.magma_dxgesv_vbatched_work(900, None, None, c["max_n"], self.nrhs, None, None,
                                            None, None, None, None, None, None, None,
                                            self.itermax, self.tol, 0, None, C.byref(lw), b, None)
        if rc != 0:
            raise RuntimeError(f"workspace query returned {rc}")
        c["work"] = torch.empty((lw.value,), dtype=torch.uint8, device=dev)
        c["lwork"] = C.c_size_t(lw.value)
        stream = torch.cuda.Stream(dev)
        c["gq"] = Queue(dev.index, stream.cuda_stream)
        torch.cuda.synchronize(dev)
        with torch.cuda.stream(stream):
            self._calls(c, c["gq"])               # eager once (kernel attributes)
            stream.synchronize()
            n0 = lib.magma_lu_launch_count()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                self._calls(c, c["gq"])
            self.graph_kernels_per_step = lib.magma_lu_launch_count() - n0
        c["graph"] = g
        torch.cuda.synchronize(dev)
        return c

    def step(self, c, i):
        if getattr(self, "eager", False):         # --profile --eager: the same calls, no graph
            self._calls(c, c["gq"])
        else:
            c["graph"].replay()

    # End to end: the batch as two halves, each with its own buffers and captured graph; the
    # second half's inputs arrive on a copy stream while the first half's graph runs, and each
    # half's solutions and gradients go back as soon as its graph is done.  (Measured on
    # GB300: 37.6 ms per step, 40.7 as one graph.)
    E2E_HALVES = 2

    def e2e_setup(self, c):
        import torch
        dev = c["A"].buf.device
        ns, As, Bs, Gs = c["ns"], c["As"], c["Bs"], c["Gs"]
        h = len(ns) // 2
        c["e2e_halves"] = []
        h2d = d2h = 0
        for lo, hi in ((0, h), (h, len(ns))):
            hc = self._context(dev, c["lib"], ns[lo:hi], As[lo:hi], Bs[lo:hi], Gs[lo:hi])
            for k in ("A", "B", "G"):
                hc["h" + k] = hc[k].buf.cpu().pin_memory()
            for k in ("X", "GB", "GA"):
                hc["h" + k] = torch.empty_like(hc[k].buf, device="cpu").pin_memory()
            h2d += (hc["hA"].numel() + hc["hB"].numel() + hc["hG"].numel()) * 8
            d2h += (hc["hX"].numel() + hc["hGB"].numel() + hc["hGA"].numel()) * 8
            c["e2e_halves"].append(hc)
        c["copy_stream"] = torch.cuda.Stream(dev)
        return h2d, d2h

    def e2e_step(self, c):
        import torch
        main, cs = torch.cuda.current_stream(), c["copy_stream"]
        cs.wait_stream(main)                      # the previous step is done with the buffers
        arrived = []
        with torch.cuda.stream(cs):
            for hc in c["e2e_halves"]:
                for k in ("A", "B", "G"):
                    hc[k].buf.copy_(hc["h" + k], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                arrived.append(ev)
        for hc, ev in zip(c["e2e_halves"], arrived):
            main.wait_event(ev)
            hc["graph"].replay()
            done = torch.cuda.Event()
            done.record(main)
            with torch.cuda.stream(cs):
                cs.wait_event(done)
                for k in ("X", "GB", "GA"):
                    hc["h" + k].copy_(hc[k].buf, non_blocking=True)
        main.wait_stream(cs)                      # the step ends when the results are home

    def accuracy(self, c, last):
        """Forward scaled residual ||B - A X|| / (||A|| ||X|| n eps) and adjoint scaled residual
        ||G - A^T GB|| / (||A^T|| ||GB|| n eps); a solve counts when both are <= 30."""
        import torch
        ok, worst_f, worst_b = 0, 0.0, 0.0
        dev = c["A"].buf.device
        for k, n in enumerate(c["ns"]):
            A = torch.from_numpy(c["As"][k]).to(dev).T          # math orientation
            X = c["X"].view(k).T
            B = torch.from_numpy(c["Bs"][k]).to(dev).T
            GB = c["GB"].view(k).T
            G = torch.from_numpy(c["Gs"][k]).to(dev).T
            rf = float(scaled_residuals(A[None], X[None], B[None])[0])
            rb = float(scaled_residuals(A.T[None], GB[None], G[None])[0])
            worst_f, worst_b = max(worst_f, rf), max(worst_b, rb)
            ok += rf <= 30 and rb <= 30
        it = c["iter"].cpu().numpy()
        ia = c["iter_adj"].cpu().numpy()
        return ok, max(worst_f, worst_b), {
            "max_scaled_residual_forward": worst_f, "max_scaled_residual_adjoint": worst_b,
            "iterations_forward": {str(int(k)): int(v) for k, v in zip(*np.unique(it, return_counts=True))},
            "iterations_adjoint": {str(int(k)): int(v) for k, v in zip(*np.unique(ia, return_counts=True))}}

    def fp64_path(self, c, steps, warmup):
        """Plain FP64: magma_dgesv_vbatched, then magma_dgetrs_vbatched(MagmaTrans) with its
        factors and magmablas_dger_neg_vbatched, on private copies of the same inputs."""
        import torch
        from magma_gb300.batched import VBatch, Queue
        lib, b, ns = c["lib"], self.batch, c["ns"]
        dev = c["A"].buf.device
        q = Queue.current(dev)
        stream = torch.cuda.current_stream(dev)
        A = VBatch(c["A"].shapes, ns, torch.float64, dev)
        X = VBatch(c["B"].shapes, ns, torch.float64, dev)
        GB = VBatch(c["G"].shapes, ns, torch.float64, dev)
        GA = VBatch(c["GA"].shapes, ns, torch.float64, dev)
        ipiv = torch.zeros((sum(ns),), dtype=torch.int32, device=dev)
        offs = np.concatenate([[0], np.cumsum(ns)[:-1]])
        dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=dev) * 4
        info = torch.empty((b,), dtype=torch.int32, device=dev)

        def call():
            A.buf.copy_(c["A"].buf)
            X.buf.copy_(c["B"].buf)
            GB.buf.copy_(c["G"].buf)
            rc = lib.magma_dgesv_vbatched(vp(A.ncols), vp(X.ncols), vp(A.ptrs), vp(A.ld), vp(dP),
                                          vp(X.ptrs), vp(X.ld), vp(info), b, q.handle)
            rc = rc or lib.magma_dgetrs_vbatched(112, vp(A.ncols), vp(GB.ncols), vp(A.ptrs),
                                                 vp(A.ld), vp(dP), vp(GB.ptrs), vp(GB.ld), b,
                                                 q.handle)
            rc = rc or lib.magmablas_dger_neg_vbatched(vp(A.ncols), vp(GB.ncols), c["max_n"],
                                                       vp(GB.ptrs), vp(GB.ld), vp(X.ptrs),
                                                       vp(X.ld), vp(GA.ptrs), vp(GA.ld), b,
                                                       q.handle)
            if rc != 0:
                raise RuntimeError(f"plain FP64 variable-size path returned {rc}")
        for _ in range(warmup):
            call()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            call()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        ok = 0
        for k in range(b):
            Am = torch.from_numpy(c["As"][k]).to(dev).T
            rf = float(scaled_residuals(Am[None], X.view(k).T[None],
                                        torch.from_numpy(c["Bs"][k]).to(dev).T[None])[0])
            rb = float(scaled_residuals(Am.T[None], GB.view(k).T[None],
                                        torch.from_numpy(c["Gs"][k]).to(dev).T[None])[0])
            ok += rf <= 30 and rb <= 30
        return {"value": ok / (ms * 1e-3), "unit": "solves/s", "ms_per_step": ms, "steps": steps,
                "note": "includes restoring the inputs (three device copies) each step",
                "call": "magma_dgesv_vbatched + magma_dgetrs_vbatched(MagmaTrans) + "
                        "magmablas_dger_neg_vbatched"}

    def roofline(self, kern, peaks, c):
        # the step is one graph replay; its FP32 factorisation (2/3 n^3 per matrix) is the
        # largest block of work, reported against the FP32 FMA rate, and the FP64 residual
        # passes against the FP64 rate
        import torch
        ms = kern["launch_ms"]
        flops = self.flops()
        ach = flops / (ms * 1e-3) / 1e12
        return {"bound": "fp32", "achieved": ach, "peak": peaks["fp32_tflops"], "unit": "TFLOP/s",
                "frac": ach / peaks["fp32_tflops"], "traffic": None, **kern,
                "kernel": "one CUDA-graph replay (factorisation flops / replay time)",
                "algorithmic_flops_per_launch": flops,
                "peak_source": "FP32 FMA-throughput probe run inside bench.py"}

    def cpu_sample(self, nthreads, target_s):
        ns, As, Bs, Gs = self.host_inputs() if not hasattr(self, "_host") else self._host
        self._host = (ns, As, Bs, Gs)

        def run(k):
            a = [x.copy() for x in As[:k]]
            b = [x.copy() for x in Bs[:k]]
            g = [x.copy() for x in Gs[:k]]
            t0 = time.perf_counter()
            cpu_adjoint_list(ns[:k], [self.nrhs] * k, a, b, g, nthreads)
            return time.perf_counter() - t0
        k = 16
        t = run(k)
        k = int(min(self.batch, max(k, k * target_s / max(t, 1e-6))))
        ts = [run(k) for _ in range(3)]
        return k, statistics.median(ts), f"the first {k} of the {self.batch} matrices (FP64 " \
                                         f"dgetrf + dgetrs + transposed dgetrs + outer product)"


class Routine:
    """--profile only: one of the routines beside the LU path (Cholesky solve, batched
    inverse, LU without pivoting, RBT solve) on `batch` FP64 matrices of order n with
    4 right-hand sides, so that their kernels can be captured at a realistic size:
    --workload posv|getri|gesv_nopiv|gesv_rbt [--batch B] (default 512 matrices,
    n = 256)."""
    n, nrhs = 256, 4

    def __init__(self, name):
        self.name = name
        self.batch = 512

    def setup(self, dev, nsteps, lib, q):
        import torch
        from magma_gb300.batched import ptr_array
        g = torch.Generator(device="cpu").manual_seed(7)
        b, n, r = self.batch, self.n, self.nrhs
        A = torch.rand((b, n, n), generator=g, dtype=torch.float64) * 2 - 1
        if self.name == "posv":
            A = A @ A.transpose(1, 2) + n * torch.eye(n, dtype=torch.float64)
        elif self.name == "gesv_nopiv":
            A = A + n * torch.eye(n, dtype=torch.float64)     # diagonally dominant
        S0 = A.transpose(1, 2).contiguous().to(dev)
        B0 = (torch.rand((b, r, n), generator=g, dtype=torch.float64) * 2 - 1).to(dev)
        c = {"lib": lib, "q": q, "S0": S0, "B0": B0, "S": S0.clone(), "B": B0.clone(),
             "info": torch.empty((b,), dtype=torch.int32, device=dev)}
        c["dS"], c["dB"] = ptr_array(c["S"]), ptr_array(c["B"])
        if self.name == "getri":
            c["inv"] = torch.empty_like(S0)
            c["dI"] = ptr_array(c["inv"])
            c["ipiv"] = torch.empty((b, n), dtype=torch.int32, device=dev)
            c["dP"] = ptr_array(c["ipiv"])
            rc = lib.magma_dgetrf_batched(n, n, vp(c["dS"]), n, vp(c["dP"]), vp(c["info"]), b, q.handle)
            if rc != 0:
                raise RuntimeError(f"magma_dgetrf_batched returned {rc}")
        return c

    def step(self, c, i):
        lib, q, b, n, r = c["lib"], c["q"], self.batch, self.n, self.nrhs
        if self.name != "getri":
            c["S"].copy_(c["S0"])
            c["B"].copy_(c["B0"])
        if self.name == "posv":
            rc = lib.magma_dposv_batched(122, n, r, vp(c["dS"]), n, vp(c["dB"]), n, vp(c["info"]), b,
                                         q.handle)
        elif self.name == "getri":
            rc = lib.magma_dgetri_outofplace_batched(n, vp(c["dS"]), n, vp(c["dP"]), vp(c["dI"]), n,
                                                     vp(c["info"]), b, q.handle)
        elif self.name == "gesv_nopiv":
            rc = lib.magma_dgesv_nopiv_batched(n, r, vp(c["dS"]), n, vp(c["dB"]), n, vp(c["info"]), b,
                                               q.handle)
        else:
            rc = lib.magma_dgesv_rbt_batched(n, r, vp(c["dS"]), n, vp(c["dB"]), n, vp(c["info"]), b,
                                             q.handle)
        if rc != 0:
            raise RuntimeError(f"{self.name} returned {rc}")


WORKLOADS = {"dsgesv512": Dsgesv512, "gesv32": Gesv32, "vbatched4096": GesvVbatched,
             "adjoint2048": Adjoint2048, "serve256": Serve256}
ROUTINES = ("posv", "getri", "gesv_nopiv", "gesv_rbt")


# DRAM bytes (read + write) per unit of work of each workload's dominant kernel, from the ncu
# captures summarised in profiles/ (a unit: one matrix, or one matrix-pass of the residual).
TRAFFIC = {
    "dsgesv512": {
        "kernel": "mlu::ir_residual_kernel<4>", "unit": "matrix-pass (n=512, nrhs=4)",
        "dram_bytes_per_unit": 276043776 / 128,
        "note": "ncu capture of the first residual pass of a 128-matrix case (every matrix "
                "active): dram__bytes_read.sum 272.84 MB + dram__bytes_write.sum 3.20 MB for 128 "
                "matrix-passes, scaled by the residual passes of the step "
                "(profiles/ir_residual_kernel_fp64_n512_batch128.md)"},
    "gesv32": {
        "kernel": "mlu::small_gesv_kernel<double,32,1>", "unit": "matrix (n=32, nrhs=1)",
        "dram_bytes_per_unit": 110.8e6 / 10000,
        "note": "ncu capture of one launch over 10,000 matrices: 84.9 MB read + 25.8 MB written "
                "(profiles/small_gesv_kernel_fp64_n32_batch10000.md)"},
}


def _traffic(name):
    return TRAFFIC.get(name)


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


class KernelTimer:
    """CUDA-event timing of one kernel class inside the library (magma_lu_timing_start /
    magma_lu_timing_stop): events on the launching stream around each launch."""

    def __init__(self, lib, cls):
        from magma_gb300.lib import KERNEL_CLASSES
        self.lib = lib
        self.cls = cls
        self.id = KERNEL_CLASSES[cls] if cls else None

    def start(self):
        if self.id is not None:
            rc = self.lib.magma_lu_timing_start(self.id, 1 << 16)
            if rc != 0:
                raise RuntimeError(f"magma_lu_timing_start returned {rc}")

    def stop(self, steps):
        if self.id is None:
            return None
        n, dropped, ms = C.c_int(0), C.c_int(0), C.c_double(0)
        rc = self.lib.magma_lu_timing_stop(C.byref(n), C.byref(dropped), C.byref(ms))
        if rc != 0 or n.value == 0:
            raise RuntimeError(f"magma_lu_timing_stop returned {rc}, {n.value} launches")
        return {"kernel_class": self.cls, "launches": n.value, "dropped": dropped.value,
                "steps": steps, "ms": ms.value, "launch_ms": ms.value / n.value,
                "timing": "CUDA events on the launching stream around every launch of the "
                          "class inside the timed region"}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            dist.init_process_group(backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg, dev=None):
    if pg is not None:
        if dev is not None and dev.type == "cuda":
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


def allsum(pg, x, dev):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def aggregate_rate(pg, units, ms, dev):
    """Whole-job throughput of independent replicas: the units every rank
    completed, summed, over the slowest rank's time (ms).  Returns (rate per
    second, slowest ms)."""
    total = allsum(pg, float(units), dev)
    slowest = allmax(pg, float(ms), dev)
    return total / (slowest * 1e-3), slowest


def measured_peaks(stream_handle):
    probe = C.CDLL(str(ROOT / "magma_gb300" / "libmlu_probe.so"))
    for f in ("mlu_probe_fp64_tflops", "mlu_probe_fp32_tflops"):
        getattr(probe, f).restype = C.c_double
        getattr(probe, f).argtypes = [C.c_void_p]
    p = {"fp64_tflops": probe.mlu_probe_fp64_tflops(C.c_void_p(stream_handle)),
         "fp32_tflops": probe.mlu_probe_fp32_tflops(C.c_void_p(stream_handle))}
    f = ROOT / "MEASURED_PEAKS.json"
    d = json.loads(f.read_text()) if f.exists() else {}
    p["hbm_gbs"] = d.get("hbm_gbs", 6800.0)
    p["hbm_source"] = "MEASURED_PEAKS.json" if "hbm_gbs" in d else "fallback 6800 GB/s"
    p["bf16_tflops"] = d.get("bf16_tflops", 1900.0)
    return p


# --------------------------------------------------------------------------
# CPU reference leg


def cpu_kind():
    """("lapack", description) when scipy's bundled LAPACK can be loaded: the reference's CPU
    path itself (testing/testing_zgesv_batched.cpp:160-176: lapackf77_dgesv per matrix, OpenMP
    schedule(dynamic), one BLAS thread); else ("port", ...) for the oracle's restatement."""
    from oracle import lapack
    if lapack.available():
        return "lapack", (f"LAPACK dgesv per matrix ({lapack.library_name()}, scipy's bundled "
                          f"OpenBLAS, one BLAS thread per call; the adjoint adds dgetrs('T') and "
                          f"dger), OpenMP schedule(dynamic), as testing/testing_zgesv_batched.cpp:"
                          f"160-176")
    return "port", (f"oracle/lu_oracle.c dgetrf+dgetrs per matrix (restated reference CPU path; "
                    f"scipy's LAPACK unavailable: {lapack.unavailable_reason()}), OpenMP "
                    f"schedule(dynamic)")


def cpu_threads():
    from oracle import lapack
    import oracle
    return lapack.max_threads() if lapack.available() else oracle.max_threads()


def cpu_gesv(S, X, nthreads):
    """(batch, n, ld) / (batch, nrhs, ldb) FP64 column-major, in place, on the CPU path."""
    from oracle import lapack
    if lapack.available():
        return lapack.dgesv_batched(S, X, nthreads=nthreads)
    import oracle
    return oracle.dgesv_batched(S, X, nthreads=nthreads)[1]


def cpu_gesv_list(ns, rs, As, Bs, nthreads):
    from oracle import lapack
    if lapack.available():
        return lapack.dgesv_list(As, Bs, nthreads=nthreads)
    import oracle
    return oracle.dgesv_vbatched(ns, rs, As, Bs, nthreads=nthreads)[1]


def cpu_adjoint_list(ns, rs, As, Bs, Gs, nthreads):
    """Forward solve, transposed solve and the outer product per matrix."""
    from oracle import lapack
    if lapack.available():
        GAs = [np.empty_like(a) for a in As]
        return lapack.dgesv_adjoint_list(As, Bs, Gs, GAs, nthreads=nthreads)
    import oracle
    pivs, info = oracle.dgesv_vbatched(ns, rs, As, Bs, nthreads=nthreads)
    for j in range(len(As)):
        oracle.gesv_adjoint_batched(As[j][None], pivs[j][None], Bs[j][None], Gs[j][None].copy(),
                                    nthreads=1)
    return info


def cpu_baseline(wl, target_s=3.0):
    nthreads = cpu_threads()
    kind, how = cpu_kind()
    k, t, what = wl.cpu_sample(nthreads, target_s)
    return {"value": k / t, "unit": "solves/s", "cores": nthreads, "kind": kind,
            "sample": f"{what}: {how}, {nthreads} threads, median of 3 passes"}


def run_reference(args, wl):
    world, rank, local, pg = dist_setup()
    if rank != 0:
        return 0
    nthreads = cpu_threads()
    kind, how = cpu_kind()
    k, t_probe, what = wl.cpu_sample(nthreads, target_s=2.0)
    vals = []
    for _ in range(args.warmup):
        wl.cpu_sample(nthreads, target_s=0.2)
    times = []
    for _ in range(args.steps):
        k2, t, _ = wl.cpu_sample(nthreads, target_s=max(0.5, 2.0 / max(args.steps, 1)))
        times.append((k2, t))
    tot_k = sum(k2 for k2, _ in times)
    tot_t = sum(t for _, t in times)
    value = tot_k / tot_t
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": wl.describe(), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nthreads, "kind": kind,
                             "sample": f"each step: a bounded sample of the workload ({what}); "
                                       f"{how}, {nthreads} host threads"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------
# GPU leg


def gpu_local_cpus(index):
    """Host CPUs local to GPU `index` (its PCI device's local_cpulist), or None.  The bench
    runs on them so that the pinned host buffers of the end-to-end leg sit on the GPU's
    memory node."""
    try:
        out = subprocess.run(["nvidia-smi", f"--id={index}", "--query-gpu=pci.bus_id",
                              "--format=csv,noheader"], capture_output=True, text=True,
                             timeout=20).stdout.strip().lower()
        dom, rest = out.split(":", 1)
        path = Path(f"/sys/bus/pci/devices/{int(dom, 16):04x}:{rest}/local_cpulist")
        cpus = set()
        for part in path.read_text().strip().split(","):
            lo, _, hi = part.partition("-")
            cpus.update(range(int(lo), int(hi or lo) + 1))
        return sorted(cpus) or None
    except Exception:
        return None


def run_ours(args, wl):
    import torch
    from magma_gb300 import lib as L
    from magma_gb300.batched import Queue

    world, rank, local, pg = dist_setup()
    cpus = gpu_local_cpus(local)
    if cpus:
        try:
            os.sched_setaffinity(0, cpus)
        except Exception:
            cpus = None
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = L.load()
    stream = torch.cuda.current_stream(dev)
    q = Queue.current(dev)
    nsteps = args.warmup + args.steps
    c = wl.setup(dev, nsteps, lib, q)

    for i in range(args.warmup):
        wl.step(c, i)
    torch.cuda.synchronize(dev)
    if args.profile:
        # the steps inside an NVTX range "bench_step", so that a profiler can take
        # only them (ncu --nvtx --nvtx-include "bench_step/")
        for k in range(args.steps):
            torch.cuda.nvtx.range_push("bench_step")
            wl.step(c, args.warmup + k)
            torch.cuda.synchronize(dev)
            torch.cuda.nvtx.range_pop()
        return 0

    peaks = measured_peaks(stream.cuda_stream)
    torch.cuda.synchronize(dev)
    clocks = Clocks(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier(pg, dev)
    torch.cuda.synchronize(dev)
    tracer = KernelTimer(lib, wl.dominant_class)
    tracer.start()
    n_launch0 = lib.magma_lu_launch_count()
    clocks.start()
    time.sleep(0.3)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        wl.step(c, args.warmup + k)
        ev[k][1].record(stream)
    end.record(stream)
    torch.cuda.synchronize(dev)
    barrier(pg, dev)
    clk = clocks.stop()
    launches = lib.magma_lu_launch_count() - n_launch0 + \
        getattr(wl, "graph_kernels_per_step", 0) * args.steps
    kern = tracer.stop(args.steps)
    step_ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in ev)
    acc = wl.accuracy(c, nsteps - 1)
    n_ok, max_res = acc[0], acc[1]
    extra = acc[2] if len(acc) > 2 else {}
    # solves that met the bar on every rank, per second of the slowest rank's step
    value, ms = aggregate_rate(pg, n_ok * args.steps, start.elapsed_time(end), dev)
    ms_per_step = ms / args.steps

    # device time per kernel class, one class per extra call (outside the timed region)
    breakdown = {}
    if getattr(wl, "breakdown_classes", None) and not getattr(args, "no_breakdown", False):
        i_extra = nsteps - 1
        for cls in wl.breakdown_classes:
            wl.restore(c, i_extra)
            torch.cuda.synchronize(dev)
            kt = KernelTimer(lib, cls)
            kt.start()
            wl.step(c, i_extra)
            try:
                kk = kt.stop(1)
            except RuntimeError:          # no launch of this class in the call
                kk = None
            breakdown[cls] = kk["ms"] if kk else 0.0
        wl.restore(c, i_extra)
        torch.cuda.synchronize(dev)

    # end to end through the C ABI with pinned host buffers
    h2d, d2h = wl.e2e_setup(c)
    for _ in range(max(args.warmup, 1)):
        wl.e2e_step(c)
    torch.cuda.synchronize(dev)
    barrier(pg, dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        wl.e2e_step(c)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_value, e2e_ms = aggregate_rate(pg, wl.batch * args.steps, e0.elapsed_time(e1), dev)
    e2e_ms /= args.steps

    fp64 = wl.fp64_path(c, max(2, min(args.steps, 5)), min(args.warmup, 3)) \
        if hasattr(wl, "fp64_path") else None

    if rank != 0:
        return 0
    cpu = cpu_baseline(wl) if world == 1 else None
    if kern is None:
        kern = {"kernel_class": None, "launches": args.steps, "steps": args.steps,
                "ms": step_ms * args.steps, "launch_ms": step_ms}
    kern["kernel"] = wl.dominant
    roof = wl.roofline(kern, peaks, c)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype,
        "data": "synthetic", "config": wl.describe(),
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "solves/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                "calls_per_step": (len(wl.E2E_SPLITS) if hasattr(wl, "E2E_SPLITS")
                                   else getattr(wl, "E2E_HALVES", 1)),
                "streams": getattr(wl, "E2E_STREAMS", 1),
                "host_cpus": f"{len(cpus)} GPU-local cores" if cpus else "unpinned"},
        "gpu_launches": launches,
        "clocks": clk,
        "accuracy": {"max_scaled_residual": max_res, "solves_within_30": n_ok, "of": wl.batch,
                     **extra},
        "peaks_measured": peaks,
    }
    if breakdown:
        line["kernel_class_ms_per_step"] = breakdown
        sec = wl.secondary_roofline(breakdown, peaks)
        if sec is not None:
            line["roofline_secondary"] = sec
    if fp64 is not None:
        line["fp64_path"] = fp64
        line["speedup_vs_fp64_path"] = value / fp64["value"] if fp64["value"] > 0 else None
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dsgesv512", choices=sorted(WORKLOADS) + list(ROUTINES))
    ap.add_argument("--profile", action="store_true",
                    help="run warm-up and timed launches only (for ncu), print nothing")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp16", "bf16"],
                    help="dsgesv512: factorisation precision of the refinement")
    ap.add_argument("--solver", default="ir", choices=["ir", "gmres"],
                    help="dsgesv512: refinement solver (gmres: Magma_REFINE_IRGMSTRS)")
    ap.add_argument("--batch", type=int, default=None,
                    help="with --profile: run the workload on its first BATCH matrices "
                         "(a small case for full ncu captures)")
    ap.add_argument("--eager", action="store_true",
                    help="with --profile: call the graph-replayed workloads eagerly (for ncu)")
    args = ap.parse_args()
    if args.workload in ROUTINES:
        if not args.profile:
            ap.error(f"--workload {args.workload} is only for --profile runs (kernel captures)")
        wl = Routine(args.workload)
        if args.batch is not None:
            wl.batch = args.batch
        return run_ours(args, wl)
    wl = WORKLOADS[args.workload]()
    if args.precision != "fp32":
        if args.workload != "dsgesv512":
            ap.error("--precision applies to the dsgesv512 workload")
        wl.precision = args.precision
    if args.solver != "ir":
        if args.workload != "dsgesv512":
            ap.error("--solver applies to the dsgesv512 workload")
        wl.solver = args.solver
        wl.itermax = 10     # the reference's outer limit for Magma_REFINE_IRGMSTRS at n = 512
    if args.batch is not None:
        if not args.profile:
            ap.error("--batch is only for --profile runs")
        wl.batch = args.batch
    wl.profile = args.profile
    if args.eager:
        if not args.profile or args.workload not in ("vbatched4096", "serve256"):
            ap.error("--eager is only for --profile runs of the graph-replayed workloads")
        wl.eager = True
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_ours(args, wl)


if __name__ == "__main__":
    sys.exit(main())
