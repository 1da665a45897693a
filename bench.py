#!/usr/bin/env python3
"""Benchmark: Lloyd iterations/s on the dense 4M x 128, k=1024 Gaussian-mixture workload,
with one sub-line per other configuration of the clustering hot path.

A step of the headline is one Lloyd iteration (centroid update + hard assignment) over all
4M rows in BF16 tensor-core form.

* value: device-resident rows/centers (torch tensors handed to the C ABI), K steps timed
  with CUDA events on the library's stream, barrier + synchronize on both sides.  The rows
  (2 GiB f32 + 1 GiB bf16 copy) exceed the 129 MB L2, so no flush is needed between steps.
* e2e: the reference-facing call (mc_hcluster through minicore_gb300.hcluster) with host
  buffers in pinned memory: each call uploads the rows and runs 10 Lloyd updates from the
  kmeans++ centers, then reads back centers / assignments / costs.  Copy bytes are given
  per Lloyd iteration (one tenth of a call) and per call.
* roofline: the assignment kernel (the dominant launch), from CUDA events around it.
* cpu_baseline / --impl reference: the oracle (C++/OpenMP restatement of the reference's
  CPU path) on a 50,000-row sample, one assignment + one centroid update per iteration,
  median of repeats, scaled to the full row count.  The in-line cpu_baseline runs the
  reference arm itself in a child process (no GPU work, no torch threads beside it).
* configs: the other workloads of the path, each measured in the same run with its own
  roofline, CPU baseline, end-to-end call from host buffers, clocks and an FP64 accuracy
  block: C1 (10,000 x 50, k = 25, whole hcluster calls), C2 (CSR 1M x 20,000, MKL and JSD,
  k = 50), C3 in TF32, C4 (coreset pipeline on 2M x 64).  C5 (serving) runs a 1000-job
  stream; `--workload serving` runs the full 20,000-job stream.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, D, K, COMPONENTS = 4_000_000, 128, 1024, 1024
E2E_ITERS = 10
CPU_SAMPLE = 50_000          # rows of the dense CPU-baseline sample
CSR_D, CSR_NNZ_ROW, CSR_K = 20_000, 1500, 50


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16", choices=["bf16", "tf32", "fp32"])
    ap.add_argument("--n", type=int, default=N)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the C1/C2/C3-TF32/C4 sub-lines of the default run")
    ap.add_argument("--workload", default="dense", choices=["dense", "csr_mkl", "csr_jsd", "csr_l1", "serving", "coreset",
                                                         "pcmp", "minibatch", "soft", "small", "coreset_mb", "tf32"],
                    help="dense: the 4M x 128 k=1024 Lloyd workload with every config as a sub-line (the default "
                         "line); csr_*: the sparse count-data workload (1M x 20000, 1500 nnz/row, k=50); serving: "
                         "the Poisson job stream through the continuous-batching server; coreset: the 2M x 64 "
                         "kmeans++ -> sensitivity -> sampling -> weighted Lloyd pipeline; small: 10000 x 50; "
                         "tf32: the 4M x 128 workload in TF32")
    ap.add_argument("--coreset-rows", type=int, default=2_000_000)
    ap.add_argument("--serving-jobs", type=int, default=20000,
                    help="jobs in the --workload serving stream (the full stream is 20000)")
    ap.add_argument("--serving-rate", type=float, default=200.0)
    ap.add_argument("--slots", type=int, default=16)
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the short serving run (p50/p99 job latency) in the default line")
    ap.add_argument("--csr-rows", type=int, default=1_000_000)
    ap.add_argument("--cpu-sample", type=int, default=CPU_SAMPLE)
    return ap.parse_args(argv)


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during a timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except Exception:
            self.proc.kill()
        s = [x for x in self.samples if len(x) >= 8]
        if not s:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(x[0]) for x in s if x[0].replace(".", "").isdigit()]
        mx = [float(x[1]) for x in s if x[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for x in s for i in range(4) if x[4 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(s)}


def replica_throughput(ms_local, steps, world, device):
    """Independent replicas (one per rank, no collective on the data path): the slowest
    rank's time bounds the job, and every rank completed `steps` iterations.  Returns
    (ms per step, whole-job iterations per second)."""
    ms = float(ms_local)
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / steps
    return ms_per_step, world * 1000.0 / ms_per_step


class Env:
    """The library, a context and the non-default stream it launches on (CUDA events that
    time a region are recorded on the same stream)."""

    def __init__(self, device=0):
        import torch
        import minicore_gb300 as mc
        from minicore_gb300 import _lib
        torch.cuda.set_device(device)
        self.torch, self.mc, self._lib = torch, mc, _lib
        self.lib = _lib.load()
        self.ctx = mc.Context(device)
        self.stream = torch.cuda.Stream()
        torch.cuda.set_stream(self.stream)
        self.ctx.set_stream(self.stream.cuda_stream)

    def event(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e

    def timed(self, fn, steps, warmup=0, profile=False):
        """warmup + steps calls of fn; returns (ms per call, kernel launches per call,
        library phases {name: {count, ms}} over the timed calls, clocks)."""
        torch, lib = self.torch, self.lib
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        clk = Clocks().start()
        if profile:
            lib.mc_profile_reset()
            lib.mc_profile_enable(1)
        l0 = lib.mc_kernel_launches()
        e0 = self.event()
        for _ in range(steps):
            fn()
        e1 = self.event()
        torch.cuda.synchronize()
        launches = int(lib.mc_kernel_launches() - l0)
        clocks = clk.stop()
        phases = {}
        if profile:
            lib.mc_profile_enable(0)
            buf = ctypes.create_string_buffer(1 << 16)
            self._lib.check(lib.mc_profile_report(buf, len(buf)))
            phases = json.loads(buf.value.decode())
        return e0.elapsed_time(e1) / steps, launches / max(steps, 1), phases, clocks

    def free(self):
        self.torch.cuda.synchronize()
        self.torch.cuda.empty_cache()


def kernel_ms(phases, *names):
    """(ms per launch, launches) of the first phase present among `names`."""
    for nm in names:
        p = phases.get(nm)
        if p and p.get("count"):
            return p["ms"] / p["count"], p["count"]
    return float("nan"), 0


# ------------------------------------------------------------------------------------
# synthetic inputs (seeded; the reference's benchmark datasets are not available)
# ------------------------------------------------------------------------------------
def make_data(n, seed=0):
    """1024 component means ~N(0, 4I), points ~N(mean, I) (seeded, generated on the GPU)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    mu = torch.randn(COMPONENTS, D, generator=g, device="cuda") * 2.0
    lab = torch.randint(0, COMPONENTS, (n,), generator=g, device="cuda")
    X = torch.randn(n, D, generator=g, device="cuda")
    X.add_(mu[lab])
    return X.contiguous()


def make_csr_counts(n, d=CSR_D, nnz_row=CSR_NNZ_ROW, seed=0, chunk=4096):
    """CSR count matrix: per row nnz_row distinct columns drawn by Zipf(1.1) rank weights
    without replacement (Gumbel top-k on the log weights, columns ranked by a seeded
    permutation); values negative binomial (mean 3, dispersion 0.5: r = 2) with zeros
    redrawn.  Generated on the GPU in row chunks; returns (values, indices, indptr)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    rank = torch.randperm(d, generator=g, device="cuda").float() + 1.0
    logw = -1.1 * torch.log(rank)
    vals = torch.empty(n * nnz_row, dtype=torch.float32, device="cuda")
    idx = torch.empty(n * nnz_row, dtype=torch.int32, device="cuda")
    for r0 in range(0, n, chunk):
        r1 = min(n, r0 + chunk)
        m = r1 - r0
        u = torch.rand((m, d), generator=g, device="cuda").clamp_(1e-12, 1.0)
        key = logw[None, :] - torch.log(-torch.log(u))
        top = torch.topk(key, nnz_row, dim=1, sorted=False).indices
        top, _ = torch.sort(top, dim=1)
        # NB(mean 3, r=2): Poisson(Gamma(shape 2, scale 1.5)), zeros redrawn
        lam = torch._standard_gamma(torch.full((m, nnz_row), 2.0, device="cuda"), generator=g) * 1.5
        x = torch.poisson(lam, generator=g)
        for _ in range(64):
            z = x == 0
            if not bool(z.any()):
                break
            lam2 = torch._standard_gamma(torch.full((int(z.sum()),), 2.0, device="cuda"), generator=g) * 1.5
            x[z] = torch.poisson(lam2, generator=g)
        x.clamp_(min=1.0)
        vals[r0 * nnz_row:r1 * nnz_row] = x.reshape(-1)
        idx[r0 * nnz_row:r1 * nnz_row] = top.reshape(-1).int()
    indptr = torch.arange(0, n + 1, device="cuda", dtype=torch.int64) * nnz_row
    return vals, idx, indptr


def make_coreset_data(n, d=64, comps=200, seed=0):
    """200 means ~N(0, 4I); component weights ~Dirichlet(0.3); 2M points ~N(mean, I)."""
    import torch
    rng = np.random.default_rng(seed)
    wts = torch.from_numpy(rng.dirichlet(np.full(comps, 0.3))).cuda()
    g = torch.Generator(device="cuda").manual_seed(seed)
    mu = torch.randn(comps, d, generator=g, device="cuda") * 2.0
    lab = torch.multinomial(wts, n, replacement=True, generator=g)
    return torch.randn(n, d, generator=g, device="cuda").add_(mu[lab]).contiguous()


def make_small_data(seed=0):
    """10,000 x 50: 25 centers ~U[-10, 10]^50, 400 points each ~N(center, I), shuffled."""
    rng = np.random.default_rng(seed)
    mu = rng.uniform(-10, 10, (25, 50))
    return (mu[rng.integers(0, 25, 10000)] + rng.normal(size=(10000, 50))).astype(np.float32)


def pinned_copy(t):
    """A pinned host copy of a device tensor (the host buffers of the end-to-end calls)."""
    import torch
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t)
    return h


def pinned_h2d_rate(h, nbytes=1 << 29):
    """This box's pinned host -> device copy rate (GB/s, best of two 512 MB copies, CUDA
    events): the end-to-end calls' upload runs at it, and it varies from box to box."""
    import torch
    flat = h.reshape(-1).view(torch.uint8)[:nbytes]
    dev = torch.empty(flat.shape, dtype=torch.uint8, device="cuda")
    best = 0.0
    for _ in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        dev.copy_(flat, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, flat.numel() / (e0.elapsed_time(e1) * 1e-3) / 1e9)
    del dev
    return best


# ------------------------------------------------------------------------------------
# accuracy against FP64 (numpy / scipy in float64)
# ------------------------------------------------------------------------------------
def fp64_sqrl2_check(Xs, C, asn_s, costs_s):
    """SQRL2 on a row sample: FP64 distances (||x||^2 - 2 x.c + ||c||^2 in float64) to the
    same centers; the GPU's objective over the sample and its argmin agreement."""
    Xs = np.asarray(Xs, np.float64)
    C64 = np.asarray(C, np.float64)
    cn = (C64 * C64).sum(1)
    best = np.empty(len(Xs))
    arg = np.empty(len(Xs), np.int64)
    for i in range(0, len(Xs), 8192):
        x = Xs[i:i + 8192]
        dist = (x * x).sum(1)[:, None] - 2.0 * (x @ C64.T) + cn[None, :]
        arg[i:i + 8192] = dist.argmin(1)
        best[i:i + 8192] = np.maximum(dist.min(1), 0.0)
    obj64 = float(best.sum())
    obj_gpu = float(np.asarray(costs_s, np.float64).sum())
    diff = np.nonzero(arg != asn_s)[0]
    gap = 0.0
    if len(diff):
        xd = Xs[diff]
        cd = C64[np.asarray(asn_s)[diff].astype(np.int64)]
        gap = float((((xd - cd) ** 2).sum(1) - best[diff]).max())
    return {"sample_rows": int(len(Xs)), "objective_gpu": obj_gpu, "objective_fp64": obj64,
            "rel_err": abs(obj_gpu - obj64) / max(obj64, 1e-300),
            "argmin_agreement": float(1.0 - len(diff) / max(len(Xs), 1)),
            "max_fp64_gap_where_argmin_differs": gap}


def fp64_objective_check(job, X, n, sample=100_000, seed=5):
    """After the timed steps: the job's assignment and objective on a fixed row subsample
    against FP64 distances with the same centers."""
    import torch
    k, d = job.k, X.shape[1]
    C = np.empty((k, d), np.float32)
    asn = np.empty(n, np.uint32)
    costs = np.empty(n, np.float64)
    job.read(C, asn, costs)
    S = np.sort(np.random.default_rng(seed).choice(n, min(sample, n), replace=False))
    Xs = X[torch.from_numpy(S).cuda()].cpu().numpy()
    return fp64_sqrl2_check(Xs, C, asn[S], costs[S])


def fp64_csr_distances(msr, sub, C):
    """MKL or JSD (prior 1) between every sample row and every center in float64, through
    identities that hold exactly in real arithmetic (prior 1: pv = 1, psum = d).  With
    c~ = (c + 1) / (sum c + d) and p~ = (x + 1) / (sum x + d):
      MKL:  KL(c~ || p~) = sum c~ log c~ - sum_{j in nz(x)} c~_j log(1 + x_j) + log(sum x + d)
      JSD:  1/2 sum_j f(c~_j, p~_j), f(a, b) = a log a + b log b - (a + b) log((a + b) / 2), over
            all columns: the zero columns take p~_j = r = 1 / (sum x + d), so the row's sum is
            sum_j f(c~_j, r) + sum_{j in nz} [f(c~_j, p~_j) - f(c~_j, r)]."""
    import scipy.sparse as sp
    d = sub.shape[1]
    C64 = np.asarray(C, np.float64)
    ct = (C64 + 1.0) / (C64.sum(1, keepdims=True) + d)            # k x d
    rs = np.asarray(sub.sum(1)).ravel().astype(np.float64)
    if msr == 5:
        H = (ct * np.log(ct)).sum(1)                                  # k
        L = sp.csr_matrix((np.log1p(sub.data.astype(np.float64)), sub.indices, sub.indptr), shape=sub.shape) @ ct.T
        out = H[None, :] - np.asarray(L) + np.log(rs + d)[:, None]
        return np.maximum(out, 0.0)

    def f(a, b):
        return a * np.log(a) + b * np.log(b) - (a + b) * np.log((a + b) * 0.5)

    out = np.empty((sub.shape[0], C64.shape[0]))
    for i in range(sub.shape[0]):
        b, e = sub.indptr[i], sub.indptr[i + 1]
        cols = sub.indices[b:e]
        r = 1.0 / (rs[i] + d)
        p = (sub.data[b:e].astype(np.float64) + 1.0) * r
        tot = f(ct, r).sum(1)
        a = ct[:, cols]
        tot += (f(a, p[None, :]) - f(a, r)).sum(1)
        out[i] = 0.5 * tot
    return np.maximum(out, 0.0)


def csr_accuracy(msr, sub, C, asn_g, cost_g, oasn, ocost, fp64_rows):
    """The GPU's assignment of a CSR row sample against the oracle (same FP32 arithmetic
    as the reference, FT = float) and against FP64."""
    oasn = np.asarray(oasn)
    diff = np.nonzero(asn_g != oasn)[0]
    rel = np.abs(cost_g - ocost) / np.maximum(np.abs(ocost), 1e-30)
    out = {"oracle_sample_rows": int(sub.shape[0]),
           "argmin_agreement_vs_oracle": float(1.0 - len(diff) / sub.shape[0]),
           "max_rel_cost_diff_vs_oracle": float(rel.max()),
           "disagreeing_rows": int(len(diff))}
    if len(diff):
        # the oracle's distance to the GPU's pick relative to its own best, at each disagreeing row
        D64 = fp64_csr_distances(msr, sub[diff], C)
        g = D64[np.arange(len(diff)), asn_g[diff].astype(np.int64)]
        o = D64[np.arange(len(diff)), oasn[diff].astype(np.int64)]
        out["fp64_margin_at_disagreements"] = [float((gi - oi) / max(abs(oi), 1e-30)) for gi, oi in zip(g, o)][:20]
    S = min(fp64_rows, sub.shape[0])
    D64 = fp64_csr_distances(msr, sub[:S], C)
    best = D64.min(1)
    arg = D64.argmin(1)
    obj64 = float(best.sum())
    objg = float(np.asarray(cost_g[:S], np.float64).sum())
    dg = np.nonzero(arg != asn_g[:S])[0]
    out.update({"fp64_sample_rows": int(S), "objective_gpu": objg, "objective_fp64": obj64,
                "rel_err": abs(objg - obj64) / max(obj64, 1e-300),
                "argmin_agreement": float(1.0 - len(dg) / S),
                "max_fp64_rel_gap_where_argmin_differs":
                    float(((D64[dg, asn_g[:S][dg].astype(np.int64)] - best[dg]) / np.maximum(best[dg], 1e-30)).max())
                    if len(dg) else 0.0})
    return out


# ------------------------------------------------------------------------------------
# CPU baseline (the oracle: the reference's CPU path restated, FT = float)
# ------------------------------------------------------------------------------------
def cpu_lloyd_iteration(X_sample, C, msr=2, prior=0.0, repeats=3):
    """Seconds of one oracle Lloyd iteration (assignment + centroid update) on a sample:
    the median over repeats of [assign, update, assign] minus the median of [assign]."""
    import oracle
    oracle.build()
    ta, tc = [], []
    for _ in range(repeats):
        t0 = time.perf_counter()
        oracle.assign(X_sample, C, msr, prior)
        ta.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        oracle.hcluster(X_sample, C, msr, prior, eps=0.0, maxiter=0, seed=1)
        tc.append(time.perf_counter() - t0)
    return float(np.median(tc) - np.median(ta)), float(np.median(ta))


def cpu_reference_line(steps=5, warmup=1, sample=CPU_SAMPLE):
    """The reference arm, run as a child process (no torch, no GPU in that process)."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", str(steps),
           "--warmup", str(warmup), "--cpu-sample", str(sample)]
    r = subprocess.run(cmd, capture_output=True, text=True, env={**os.environ, "RANK": "0", "WORLD_SIZE": "1"})
    for line in r.stdout.splitlines()[::-1]:
        if line.startswith("{"):
            return json.loads(line)
    return None


# ------------------------------------------------------------------------------------
# CSR L1 (prior 0)
# ------------------------------------------------------------------------------------
def csr_l1_bench(args):
    """CSR L1 (prior 0) on the sparse count workload: D^2 seeding (k=50), then the timed
    step is one L1 Lloyd iteration (sparse coordinate-wise medians of the clusters, then the
    L1 assignment pass: the union walk over nonzero columns) with rows resident in HBM."""
    import torch
    import minicore_gb300 as mc
    from minicore_gb300 import _lib
    torch.cuda.set_device(0)
    ctx = mc.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    n, d, k = args.csr_rows, 20_000, 50
    msr = {"csr_mkl": 5, "csr_jsd": 4, "csr_l1": 0}[args.workload]
    prior = 0.0 if msr == 0 else 1.0
    vals, idx, indptr = make_csr_counts(n, d, seed=0)
    torch.cuda.synchronize()
    A = mc.CSparseMatrix(data=vals, indices=idx, indptr=indptr, shape=(n, d))
    M = mc._MatrixArg(A)
    lib = _lib.load()
    u = torch.from_numpy(mc.uniforms(99, k)).cuda()
    ids = torch.empty(k, dtype=torch.int32, device="cuda")
    asn = torch.empty(n, dtype=torch.int32, device="cuda")
    costs = torch.empty(n, dtype=torch.float64, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    _lib.check(lib.mc_kmeanspp(ctx.handle, M.ref, k, msr, prior, None, mc._p(u), mc._p(ids), mc._p(asn),
                               mc._p(costs)))
    e1.record(stream)
    torch.cuda.synchronize()
    kmpp_ms = e0.elapsed_time(e1)
    C = torch.zeros((k, d), dtype=torch.float32, device="cuda")
    ipc = indptr.cpu()
    for c, r in enumerate(ids.cpu().tolist()):
        b, e = int(ipc[r]), int(ipc[r + 1])
        C[c, idx[b:e].long()] = vals[b:e]
    job = mc.Job(A, C, msr=msr, prior=prior, ctx=ctx)
    step = job.lloyd_step if msr == 0 else job.assign
    job.assign()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    lib.mc_profile_reset()
    lib.mc_profile_enable(1)
    l0 = lib.mc_kernel_launches()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    lib.mc_profile_enable(0)
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.check(lib.mc_profile_report(buf, len(buf)))
    phases = json.loads(buf.value.decode())
    launches = int(lib.mc_kernel_launches() - l0)
    ms = e0.elapsed_time(e1) / args.steps
    nnz = n * 1500
    algo_bytes = nnz * 8 + (n + 1) * 8 + n * 8 + n * 12 + k * d * 4
    pk, pk_kind = peaks()
    kern = (phases.get("assign_csr_sparse") or phases.get("assign_csr_l1_union") or phases.get("assign_csr_tiled")
            or {})
    kms = kern.get("ms", float("nan")) / max(kern.get("count", 1), 1)
    name = {5: "MKL", 4: "JSD", 0: "L1"}[msr]
    rows_tag = f"{n // 1_000_000}M" if n % 1_000_000 == 0 else f"{n // 1000}k"
    metric = (f"CSR L1 Lloyd iterations/s {rows_tag}x20000 k=50" if msr == 0
              else f"CSR {name} assignment passes/s {rows_tag}x20000 k=50")
    unit = "iters/s" if msr == 0 else "passes/s"
    out = {"metric": metric, "value": 1000.0 / ms, "unit": unit, "ms_per_pass": ms, "steps": args.steps,
           "warmup": args.warmup, "dtype": "f32", "data": "synthetic", "gpu_launches": launches,
           "config": {"workload": f"CSR {n}x{d}, 1500 nnz/row Zipf(1.1) columns, NB(3,0.5) counts, "
                                  f"msr={msr}, prior={prior:g}, k={k}, kmeans++ centers"},
           "kmeanspp_ms": kmpp_ms,
           "roofline": {"bound": "hbm" if msr == 5 else ("issue (divergent merge)" if msr == 0 else "compute"),
                        "achieved": algo_bytes / (kms * 1e-3) / 1e9,
                        "peak": pk.get("hbm_gbs", 6767.7), "unit": "GB/s",
                        "frac": algo_bytes / (kms * 1e-3) / 1e9 / pk.get("hbm_gbs", 6767.7),
                        "algorithmic_bytes": algo_bytes, "kernel_ms": kms, "peak_source": pk_kind},
           # the L1 union walk has no byte or FLOP roof: it is bound by issuing its divergent
           # integer merge (an ncu capture at 100k rows: 12.5 of 32 lanes active, 81 % issue);
           # the HBM figure above is kept for reference only
           **({"roofline_note": "L1 (prior 0): issue-bound divergent merge walk; frac against HBM is for "
                                "reference, not a bound"} if msr == 0 else {}),
           "phases_ms": phases}
    if msr != 0:
        # a whole Lloyd update (weighted means of the CSR rows, then the assignment pass),
        # the C2 loop's unit of work
        lib.mc_profile_reset()
        lib.mc_profile_enable(1)
        e0.record(stream)
        for _ in range(args.steps):
            job.lloyd_step()
        e1.record(stream)
        torch.cuda.synchronize()
        lib.mc_profile_enable(0)
        buf2 = ctypes.create_string_buffer(1 << 16)
        _lib.check(lib.mc_profile_report(buf2, len(buf2)))
        out["lloyd_step"] = {"ms": e0.elapsed_time(e1) / args.steps,
                             "iters_per_s": 1000.0 * args.steps / e0.elapsed_time(e1),
                             "phases_ms": json.loads(buf2.value.decode())}
    if msr == 0:
        # the median phase: algorithmic bytes = the nonzeros (values + indices), the row
        # pointers and assignments, and the k x d centers written
        # centroid_update: the counting sort of the rows by cluster and the medians, per step
        med = phases.get("centroid_update", {})
        med_ms = med.get("ms", float("nan")) / args.steps
        med_bytes = nnz * 8 + (n + 1) * 8 + n * 4 + k * d * 4
        out["l1_median_roofline"] = {"bound": "hbm", "achieved": med_bytes / (med_ms * 1e-3) / 1e9,
                                     "peak": pk.get("hbm_gbs", 6767.7), "unit": "GB/s",
                                     "frac": med_bytes / (med_ms * 1e-3) / 1e9 / pk.get("hbm_gbs", 6767.7),
                                     "algorithmic_bytes": med_bytes, "phase_ms": med_ms, "peak_source": pk_kind}
    if not args.no_cpu and msr == 0:
        # the oracle's assignment and sparse medians of the first S rows, scaled to n rows
        import scipy.sparse as sp
        import oracle
        S = 20000
        ipc_s = ipc[:S + 1].numpy().astype(np.int64)
        sub = sp.csr_matrix((vals[:int(ipc_s[-1])].cpu().numpy(), idx[:int(ipc_s[-1])].cpu().numpy().astype(np.int64),
                             ipc_s), shape=(S, d))
        Ch = C.cpu().numpy()
        t0 = time.perf_counter()
        a_s, _ = oracle.assign(sub, Ch, 0, 0.0)
        present = np.unique(a_s)
        remap = np.zeros(k, np.uint32)
        remap[present] = np.arange(present.size, dtype=np.uint32)
        oracle.l1_centers(sub, remap[a_s], int(present.size))
        cpu_s = (time.perf_counter() - t0) * (n / S)
        out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "iters/s", "cores": os.cpu_count() or 1,
                               "kind": "port",
                               "sample": f"oracle L1 assignment + sparse medians of the first {S} rows "
                                         f"(clusters present in the sample), scaled by {n}/{S}"}
    elif not args.no_cpu:
        # the oracle (CPU restatement, 16-thread OpenMP union walk of the reference's sparse
        # measures) on the first rows of the same matrix and centers, scaled to all n rows
        import scipy.sparse as sp
        import oracle
        S = 2000 if msr == 5 else 1000
        ipc_s = ipc[:S + 1].numpy().astype(np.int64)
        sub = sp.csr_matrix((vals[:int(ipc_s[-1])].cpu().numpy(), idx[:int(ipc_s[-1])].cpu().numpy().astype(np.int64),
                             ipc_s), shape=(S, d))
        Ch = C.cpu().numpy()
        t0 = time.perf_counter()
        oracle.assign(sub, Ch, msr, 1.0)
        cpu_s = (time.perf_counter() - t0) * (n / S)
        out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "passes/s", "cores": os.cpu_count() or 1,
                               "kind": "port",
                               "sample": f"oracle assignment of the first {S} rows against the same {k} centers, "
                                         f"scaled by {n}/{S}"}
    print(json.dumps(out))


FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12  # 152 SMs x 128 FP32 lanes x FMA x 2.07 GHz


def next_rows_bench(args):
    """Rows widened beyond the hot path, each timed with CUDA events on the library's
    stream and checked against a CPU oracle sample:
      pcmp       condensed pairwise SQRL2 distances of 20,000 x 128 rows (device output)
      minibatch  minibatch EM, 1M x 64 mixture, k = 100, mbsize 4096, 60 iterations
      soft       soft clustering, 200k x 32 mixture, k = 20, temp 1, 8 iterations"""
    import torch
    import minicore_gb300 as mc
    from minicore_gb300 import _lib
    torch.cuda.set_device(0)
    lib = _lib.load()
    ctx = mc.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    g = torch.Generator(device="cuda").manual_seed(0)

    def mixture(n, d, comps):
        mu = torch.randn(comps, d, generator=g, device="cuda") * 2.0
        lab = torch.randint(0, comps, (n,), generator=g, device="cuda")
        return torch.randn(n, d, generator=g, device="cuda").add_(mu[lab]).contiguous()

    def timed(fn, reps):
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = lib.mc_kernel_launches()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, int(lib.mc_kernel_launches() - l0)

    clocks = Clocks()
    clocks.start()
    if args.workload == "pcmp":
        n, d = 20000, 128
        X = mixture(n, d, 64)
        M = mc._MatrixArg(X)
        out = torch.empty(n * (n - 1) // 2, dtype=torch.float32, device="cuda")
        ms, launches = timed(lambda: _lib.check(lib.mc_pcmp(ctx.handle, M.ref, 2, 0.0, mc._p(out))), args.steps)
        flops = 2.0 * n * n * d  # every (row, row) pair is evaluated; half are written
        achieved = flops / (ms * 1e-3) / 1e12
        import oracle
        S = 600
        Xs = X[:S].cpu().numpy()
        t0 = time.perf_counter()
        oracle.assign(Xs, Xs, 2, 0.0)
        cpu_pairs_s = S * S / (time.perf_counter() - t0)
        line = {"metric": "condensed pairwise SQRL2 distances/s, 20000 x 128 (pcmp)",
                "value": n * (n - 1) / 2 / (ms * 1e-3), "unit": "pairs/s", "ms_per_step": ms,
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": FP32_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                             "frac": achieved / FP32_NOMINAL_TFLOPS, "traffic": None,
                             "peak_source": "nominal FP32 (152 SMs x 128 lanes x 2 x 2.07 GHz)",
                             "algorithmic": f"2*n*n*d = {flops:.4g} FLOP per call"},
                "cpu_baseline": {"value": cpu_pairs_s, "unit": "pairs/s", "cores": os.cpu_count() or 1,
                                 "kind": "port", "sample": f"oracle distances of {S} x {S} rows"}}
    elif args.workload == "coreset_mb":
        n, d, k = 1_000_000, 64, 100
        X = mixture(n, d, 200)
        ids = torch.randperm(n, generator=g, device="cuda")[:k]
        C0 = X[ids].contiguous()
        M = mc._MatrixArg(X)
        cout = torch.empty((k, d), dtype=torch.float32, device="cuda")
        asn = torch.empty(n, dtype=torch.int32, device="cuda")
        cst = torch.empty(n, dtype=torch.float64, device="cuda")
        ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()

        def run():
            _lib.check(lib.mc_hcluster_coreset(ctx.handle, M.ref, mc._p(C0), k, 2, 0.0, None, 4096, 20, 5, 1, 5,
                                               mc._PREC["bf16"], mc._p(cout), mc._p(asn), mc._p(cst),
                                               ctypes.byref(ic), ctypes.byref(fc), ctypes.byref(it)))
        ms, launches = timed(run, 1)
        line = {"metric": "coreset-minibatch EM runs/s, 1M x 64, k=100, coreset 4096, maxiter 20, 5 check-ins",
                "value": 1000.0 / ms, "unit": "runs/s", "ms_per_step": ms,
                "rounds": int(it.value), "objective": {"initcost": ic.value, "finalcost": fc.value},
                "roofline": None, "cpu_baseline": None}
    elif args.workload == "minibatch":
        n, d, k = 1_000_000, 64, 100
        X = mixture(n, d, 200)
        ids = torch.randperm(n, generator=g, device="cuda")[:k]
        C0 = X[ids].contiguous()
        iters = 60
        job = mc.Job(X, C0, msr=2, precision="bf16", seed=5, ctx=ctx)
        ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()

        def run():
            _lib.check(lib.mc_job_minibatch(job._h, 4096, iters, 10, 1, 0, ctypes.byref(ic), ctypes.byref(fc),
                                            ctypes.byref(it)))
        ms, launches = timed(run, 1)
        line = {"metric": "minibatch EM iterations/s, 1M x 64, k=100, mbsize 4096 (BF16 check-ins)",
                "value": iters / (ms * 1e-3), "unit": "iters/s", "ms_per_step": ms / iters,
                "objective": {"initcost": ic.value, "finalcost": fc.value}, "roofline": None,
                "cpu_baseline": None}
    else:
        n, d, k = 200_000, 32, 20
        X = mixture(n, d, 20)
        C0 = X[:k].contiguous()
        Xh = X.cpu().numpy()
        C0h = C0.cpu().numpy()
        M = mc._MatrixArg(X)
        iters = 8
        costs = torch.empty((n, k), dtype=torch.float32, device="cuda")
        asn = torch.empty((n, k), dtype=torch.float32, device="cuda")
        cout = torch.empty((k, d), dtype=torch.float32, device="cuda")
        ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()

        def run():
            _lib.check(lib.mc_scluster(ctx.handle, M.ref, mc._p(C0), k, 2, 0.0, None, 1.0, iters, 0.0, mc._p(cout),
                                       mc._p(costs), mc._p(asn), ctypes.byref(ic), ctypes.byref(fc),
                                       ctypes.byref(it)))
        ms, launches = timed(run, 1)
        import oracle
        S = 20000
        t0 = time.perf_counter()
        ro = oracle.scluster(Xh[:S], C0h, 2, 0.0, temp=1.0, maxiter=iters, eps=0.0)
        cpu_iter_s = (time.perf_counter() - t0) * (n / S) / max(int(ro["numiter"]), 1)
        line = {"metric": "soft clustering iterations/s, 200k x 32, k=20, temp 1",
                "value": max(int(it.value), 1) / (ms * 1e-3), "unit": "iters/s", "ms_per_step": ms / max(int(it.value), 1),
                "objective": {"initcost": ic.value, "finalcost": fc.value}, "roofline": None,
                "cpu_baseline": {"value": 1.0 / cpu_iter_s, "unit": "iters/s (scaled to 200k rows)",
                                 "cores": os.cpu_count() or 1, "kind": "port",
                                 "sample": f"oracle soft clustering of {S} rows, scaled by {n}/{S}"}}
    clk = clocks.stop()
    line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                 "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.workload != "minibatch" else "bf16",
                 "data": "synthetic", "config": {"workload": args.workload}, "gpu_launches": launches,
                 "clocks": clk, "e2e": None})
    print(json.dumps(line))


SERVE_DS = (32, 64, 128, 512)
SERVE_POOL_ROWS = 200_000


def _nb_counts(m, g):
    """m negative-binomial counts (mean 3, dispersion 0.5: Poisson(Gamma(2, 1.5))), zeros
    redrawn (a few rounds, then set to 1)."""
    import torch
    lam = torch._standard_gamma(torch.full((m,), 2.0, device="cuda"), generator=g) * 1.5
    x = torch.poisson(lam, generator=g)
    for _ in range(32):
        z = x == 0
        nz = int(z.sum())
        if nz == 0:
            break
        lam2 = torch._standard_gamma(torch.full((nz,), 2.0, device="cuda"), generator=g) * 1.5
        x[z] = torch.poisson(lam2, generator=g)
    return x.clamp_(min=1.0).float()


def make_serving_pool(seed=0, host=True):
    """Row pools the serving jobs slice: per d in {32, 64, 128, 512}, a dense 200-component
    Gaussian mixture (means ~N(0, 4I), sigma 1) and a CSR count matrix at 1% density
    (Bernoulli(0.01) columns, every row at least one entry, NB counts), 200k rows each.
    Generated on the GPU; host=True keeps pinned host copies only, so every job's rows are
    uploaded by the server under load."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    dense, csr = {}, {}
    for d in SERVE_DS:
        mu = torch.randn(200, d, generator=g, device="cuda") * 2.0
        lab = torch.randint(0, 200, (SERVE_POOL_ROWS,), generator=g, device="cuda")
        dense[d] = torch.randn(SERVE_POOL_ROWS, d, generator=g, device="cuda").add_(mu[lab]).contiguous()
        mask = torch.rand(SERVE_POOL_ROWS, d, generator=g, device="cuda") < 0.01
        force = torch.randint(0, d, (SERVE_POOL_ROWS,), generator=g, device="cuda")
        empty = (~mask.any(1)).nonzero().squeeze(1)
        mask[empty, force[empty]] = True
        rows, cols = mask.nonzero(as_tuple=True)  # row-major: columns ascending in each row
        indptr = torch.zeros(SERVE_POOL_ROWS + 1, dtype=torch.int64, device="cuda")
        indptr[1:] = torch.cumsum(torch.bincount(rows, minlength=SERVE_POOL_ROWS), 0)
        csr[d] = (_nb_counts(rows.numel(), g).contiguous(), cols.int().contiguous(), indptr)
        del mask
    if host:
        dense = {d: pinned_copy(v) for d, v in dense.items()}
        csr = {d: tuple(pinned_copy(t) for t in v) for d, v in csr.items()}
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return dense, csr


def make_serving_jobs(pool, njobs, rate, seed):
    """Seeded request stream: Poisson arrivals at `rate`/s; n log-uniform in [1e3, 2e5], d
    from {32, 64, 128, 512}, k log-uniform in [5, 200]; half dense SQRL2 in BF16 tensor-core
    form, half CSR MKL (prior 1); k-means++ seeding then Lloyd to eps 1e-4 or 10 updates."""
    import minicore_gb300 as mc
    dense, csr = pool
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, njobs)) if rate > 0 else np.zeros(njobs)
    jobs = []
    for i in range(njobs):
        n = int(np.exp(rng.uniform(np.log(1e3), np.log(2e5))))
        d = int(rng.choice(SERVE_DS))
        k = int(np.exp(rng.uniform(np.log(5), np.log(200))))
        off = int(rng.integers(0, SERVE_POOL_ROWS - n + 1))
        if rng.random() < 0.5:
            X = dense[d][off:off + n]
            spec = dict(matrix=X, k=k, msr=2, prior=0.0, precision="bf16")
            kind = "dense_sqrl2_bf16"
            h2d = n * d * 4
        else:
            v, c, ip = csr[d]
            b, e = int(ip[off]), int(ip[off + n])
            X = mc.CSparseMatrix(data=v[b:e], indices=c[b:e], indptr=(ip[off:off + n + 1] - b).contiguous(),
                                 shape=(n, d))
            spec = dict(matrix=X, k=k, msr=5, prior=1.0, precision="fp32")
            kind = "csr_mkl"
            h2d = (e - b) * 8 + (n + 1) * 8
        spec.update(eps=1e-4, maxiter=10, seed=1000 + i)
        jobs.append({"spec": spec, "t": float(arrivals[i]), "n": n, "d": d, "k": k, "kind": kind,
                     "h2d": int(h2d), "off": off})
    return jobs


def run_serving(srv, jobs, open_loop=True):
    """Submit `jobs` at their arrival times (open_loop) or all at once; returns the results
    and the wall time from the first submission to the last completion."""
    import queue
    q = queue.Queue()
    results = [None] * len(jobs)

    def collect():
        while True:
            item = q.get()
            if item is None:
                return
            i, t = item
            results[i] = srv.wait(t)

    th = threading.Thread(target=collect)
    th.start()
    t0 = time.perf_counter()
    try:
        for i, j in enumerate(jobs):
            if open_loop:
                delay = t0 + j["t"] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
            q.put((i, srv.submit(**j["spec"])))
    finally:
        q.put(None)
        th.join()
    return results, time.perf_counter() - t0


def serving_fp64_checks(pool, jobs, results, every, rows=4096):
    """Every `every`-th job's returned centers, assignment and costs against FP64, on up to
    `rows` of its rows (a fixed subsample): the objective over those rows recomputed in
    float64 (dense: squared distances; CSR MKL: the FP64 identity of fp64_csr_distances)
    against the sum of the job's returned costs there, and the argmin agreement."""
    import scipy.sparse as sp
    dense, csr = pool
    errs, agree = [], []
    for i in range(0, len(jobs), every):
        j, r = jobs[i], results[i]
        n, d, off = j["n"], j["d"], j["off"]
        S = np.sort(np.random.default_rng(i).choice(n, min(rows, n), replace=False))
        C = r["centers"]
        if j["kind"] == "csr_mkl":
            v, c, ip = csr[d]
            b, e = int(ip[off]), int(ip[off + n])
            sub = sp.csr_matrix((v[b:e].numpy(), c[b:e].numpy().astype(np.int64),
                                 (ip[off:off + n + 1] - b).numpy().astype(np.int64)), shape=(n, d))[S]
            D64 = fp64_csr_distances(5, sub, C)
            obj64 = float(D64.min(1).sum())
            ag = float((D64.argmin(1) == r["asn"][S]).mean())
        else:
            a = fp64_sqrl2_check(dense[d][off:off + n].numpy()[S], C, r["asn"][S], r["costs"][S])
            obj64, ag = a["objective_fp64"], a["argmin_agreement"]
        objg = float(np.asarray(r["costs"][S], np.float64).sum())
        errs.append(abs(objg - obj64) / max(obj64, 1e-300))
        agree.append(ag)
    return {"jobs_checked": len(errs), "rows_per_job": rows, "max_rel_err_objective_vs_fp64": float(max(errs)),
            "median_rel_err": float(np.median(errs)), "min_argmin_agreement": float(min(agree)),
            "mean_argmin_agreement": float(np.mean(agree))}


def serving_bench(njobs, rate=200.0, slots=8, seed=0, saturation_jobs=None, serial=False, check_every=100):
    """The serving form: a seeded Poisson stream of uneven jobs through mc_server (continuous
    batching over `slots` concurrent slots, admission by free device memory), rows uploaded
    from pinned host memory by the server for every job."""
    import torch
    import minicore_gb300 as mc
    from minicore_gb300 import _lib
    lib = _lib.load()
    pool = make_serving_pool(seed)
    torch.cuda.synchronize()
    jobs = make_serving_jobs(pool, njobs, rate, seed + 1)
    warm = make_serving_jobs(pool, 16, 0.0, seed + 2)
    sat = make_serving_jobs(pool, saturation_jobs or max(njobs // 4, 64), 0.0, seed + 3)
    torch.cuda.synchronize()
    out = {}
    # warm-up, untimed: the module, pools, and the autotuner's decisions for the stream's shape
    # buckets (the timed jobs then take recorded decisions, as a server with a persistent
    # tuning cache does; every job's work still runs in the timed stream)
    warm_tune = jobs[:2000]
    with mc.Server(slots=slots) as srv:
        run_serving(srv, warm, open_loop=False)
        run_serving(srv, warm_tune, open_loop=False)
        srv.reset_stats()
        clocks = Clocks().start()
        l0 = lib.mc_kernel_launches()
        res, wall = run_serving(srv, jobs, open_loop=True)
        launches = int(lib.mc_kernel_launches() - l0)
        clk = clocks.stop()
        st = srv.stats()
        srv.reset_stats()
        res_s, wall_s = run_serving(srv, sat, open_loop=False)
        st_s = srv.stats()

    def col(name, sel=None):
        a = np.array([r[name] for r in res])
        return a if sel is None else a[sel]

    def pct(a):
        return {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99)), "mean": float(a.mean())}

    rows_iters = sum(j["n"] * (r["numiter"] + 1) for j, r in zip(jobs, res))
    d2h = sum(j["k"] * j["d"] * 4 + j["n"] * 12 for j in jobs)
    h2d = sum(j["h2d"] for j in jobs)
    by_kind = {}
    tot = col("total_ms")
    for kind in ("dense_sqrl2_bf16", "csr_mkl"):
        sel = np.array([j["kind"] == kind for j in jobs])
        if sel.any():
            by_kind[kind] = {"jobs": int(sel.sum()), **{nm: pct(col(nm, sel)) for nm in
                                                        ("total_ms", "queue_ms", "setup_ms", "loop_ms", "read_ms")}}
    # the slowest 1% of jobs: their shapes and where their time went
    slow = np.argsort(tot)[-max(1, len(tot) // 100):]
    tail = {"jobs": int(len(slow)), "kinds": {k: int(sum(jobs[i]["kind"] == k for i in slow))
                                              for k in ("dense_sqrl2_bf16", "csr_mkl")},
            "median_n": float(np.median([jobs[i]["n"] for i in slow])),
            "median_k": float(np.median([jobs[i]["k"] for i in slow])),
            "median_d": float(np.median([jobs[i]["d"] for i in slow])),
            **{nm: float(np.mean(col(nm)[slow])) for nm in ("queue_ms", "setup_ms", "loop_ms", "read_ms")}}
    out = {"jobs": njobs, "rate_per_s": rate, "slots": slots, "wall_s": wall, "jobs_per_s": njobs / wall,
           "latency_ms": {"total": pct(tot), "queue": pct(col("queue_ms")), "run": pct(col("run_ms")),
                          "setup": pct(col("setup_ms")), "loop": pct(col("loop_ms")), "read": pct(col("read_ms"))},
           "server_stats": st, "by_kind": by_kind, "slowest_1pct": tail,
           "row_iterations_per_s": rows_iters / wall, "gpu_launches": launches, "clocks": clk,
           "autotune_entries": len(mc.autotune_report().get("entries", {})),
           "autotune_warmup": f"the first {len(warm_tune)} job specs of the stream run once, untimed, before it",
           "h2d_bytes": int(h2d), "d2h_bytes": int(d2h),
           "accuracy_vs_fp64": serving_fp64_checks(pool, jobs, res, check_every),
           "saturated": {"jobs": len(sat), "jobs_per_s": len(sat) / wall_s, "wall_s": wall_s,
                         "max_running": st_s.get("max_running"),
                         "latency_ms": pct(np.array([r["total_ms"] for r in res_s]))}}
    if serial:
        with mc.Server(slots=1) as srv1:
            run_serving(srv1, warm[:4], open_loop=False)
            _, wall_1 = run_serving(srv1, sat, open_loop=False)
        out["saturated_one_slot"] = {"jobs": len(sat), "jobs_per_s": len(sat) / wall_1, "wall_s": wall_1}
    return out


def serving_main(args):
    import torch
    torch.cuda.set_device(0)
    s = serving_bench(args.serving_jobs, rate=args.serving_rate, slots=args.slots, serial=True,
                      saturation_jobs=2000)
    line = {"metric": "serving jobs/s (Poisson 200/s mix of uneven clustering jobs); p50/p99 job latency",
            "value": s["jobs_per_s"], "unit": "jobs/s", "n_gpus": 1, "steps": s["jobs"], "warmup": 16,
            "ms_per_step": 1000.0 * s["wall_s"] / s["jobs"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 (dense SQRL2) / f32 (CSR MKL)", "data": "synthetic",
            "config": {"workload": f"{s['jobs']} jobs, Poisson {args.serving_rate}/s, n logU[1e3,2e5], "
                                   f"d in {{32,64,128,512}}, k logU[5,200], half dense SQRL2 BF16, half CSR "
                                   f"MKL 1% density; kmeans++ then Lloyd (eps 1e-4, 10 updates)",
                       "slots": args.slots, "rows": "pinned host pools; the server uploads every job's rows"},
            "latency_ms": s["latency_ms"], "serving": s, "gpu_launches": s["gpu_launches"],
            "clocks": s["clocks"], "accuracy_vs_fp64": s["accuracy_vs_fp64"],
            "e2e": {"value": s["jobs_per_s"], "unit": "jobs/s", "h2d_bytes_per_step": int(s["h2d_bytes"] / s["jobs"]),
                    "d2h_bytes_per_step": int(s["d2h_bytes"] / s["jobs"]),
                    "call": "minicore_gb300.Server.submit/wait (rows from pinned host memory, outputs to host)"}}
    print(json.dumps(line))


# ------------------------------------------------------------------------------------
# C3: dense 4M x 128, k = 1024 (the headline in BF16; TF32 as a sub-line)
# ------------------------------------------------------------------------------------
TC_PASS1_VARIANTS = ["k_tc_assign<{p}, TC_TOP2, BN 256, 4 stages>", "k_tc_assign<{p}, TC_TOP2, BN 256, 3 stages>",
                     "k_tc_assign<{p}, TC_TOP2, BN 128, 4 stages>", "k_tc_assign<{p}, TC_TOP2, BN 128, 6 stages>",
                     "k_tc_top2_res<{p}> (centers resident in shared memory, 2 groups of 512)"]


def tc_pass1_variant(precision, kp=1024):
    """The pass 1 kernel the autotuner kept for the 4M x 128, k = 1024 bucket (kp % 256 == 0:
    variants 0-3 are the streaming tile shapes, 4 the resident-centers kernel)."""
    import minicore_gb300 as mc
    for key, e in mc.autotune_report().get("entries", {}).items():
        if key.startswith(f"tc1|{precision}|kp{kp}|d2^7|n2^22"):
            v = int(e["variant"])
            name = TC_PASS1_VARIANTS[v] if v < len(TC_PASS1_VARIANTS) else f"variant {v}"
            return name.format(p=precision) + " (pass 1: every row x every center)", {
                "variant": v, "ms": e.get("ms")}
    return TC_PASS1_VARIANTS[0].format(p=precision) + " (pass 1: every row x every center; untuned default)", None


def tc_autotune_entries(precision, kp=1024):
    """The autotuner's decisions for the tensor-core passes of this workload's shape bucket
    (tc1: pass 1 kernel / tile shape, tc2: pass 2 tile shape), with each variant's measured
    milliseconds."""
    import minicore_gb300 as mc
    out = {}
    for key, e in mc.autotune_report().get("entries", {}).items():
        for fam in ("tc1", "tc2"):
            if key.startswith(f"{fam}|{precision}|kp{kp}|d2^7|n2^22"):
                out[fam] = {"variant": int(e["variant"]), "ms": e.get("ms")}
    return out


def tc_roofline(phases, n, precision, pk, pk_kind):
    """Pass 1 of the tensor-core assignment (every row x every center): 2 n k d FLOP per
    launch against the measured BF16 burst peak (TF32: half of it, the tensor pipe's TF32
    rate being half its BF16 rate)."""
    flops = 2.0 * n * K * D
    ms, launches = kernel_ms(phases, "tc_pass1_top2")
    kernel, variant = tc_pass1_variant(precision)
    peak = pk.get("bf16_tflops", 1935.7) * (0.5 if precision == "tf32" else 1.0)
    achieved = flops / (ms * 1e-3) / 1e12
    traffic = None
    if precision == "bf16" and n == N:
        # the ncu summary of the kernel the autotuner kept (DRAM bytes of one captured launch,
        # scaled to 4M rows)
        prof = "k_tc_top2_res_bf16_1Mx128_k1024.md" if (variant or {}).get("variant") == 4 else \
            "k_tc_assign_bf16_4Mx128_k1024.md"
        try:
            for line in open(os.path.join(ROOT, "profiles", prof)):
                if line.startswith("traffic_bytes_per_launch_scaled_to_4M:"):
                    traffic = float(line.split(":")[1].split()[0])
        except OSError:
            traffic = None
    return {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": traffic,
            "peak_source": f"{pk_kind} bf16_tflops (burst)" + (" / 2 for TF32" if precision == "tf32" else ""),
            "kernel": kernel, "autotune_variant": variant,
            "kernel_ms_per_launch": ms, "launches": launches,
            "algorithmic": f"2*n*k*d = {flops:.4g} FLOP per launch (n={n}, k={K}, d={D})"}


def dense_e2e(E, X, C0, precision, calls):
    """hcluster from pinned host rows: each call uploads the rows, runs 10 Lloyd updates and
    copies centers, assignments and costs back."""
    mc, torch = E.mc, E.torch
    n = X.shape[0]
    Xh = pinned_copy(X)
    Ch = C0.cpu().numpy()
    h2d_gbps = pinned_h2d_rate(Xh)
    mc.hcluster(Xh, Ch, msr=2, eps=0.0, maxiter=1, precision=precision, ctx=E.ctx)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    iters = 0
    for _ in range(calls):
        r = mc.hcluster(Xh, Ch, msr=2, eps=0.0, maxiter=E2E_ITERS - 1, precision=precision, ctx=E.ctx)
        iters += int(r["numiter"])
    t = time.perf_counter() - t0
    del Xh
    h2d = int(n * D * 4 + K * D * 4)
    d2h = int(K * D * 4 + n * 4 + n * 4)  # centers, assignments, float32 costs
    per_iter = iters / calls
    return {"value": iters / t, "unit": "iters/s", "h2d_bytes_per_step": int(h2d / per_iter),
            "d2h_bytes_per_step": int(d2h / per_iter), "h2d_bytes_per_call": h2d, "d2h_bytes_per_call": d2h,
            "iters_per_call": per_iter, "calls": calls,
            "pinned_h2d_gbps_this_box": h2d_gbps,
            "call": f"minicore_gb300.hcluster(pinned host rows, maxiter={E2E_ITERS - 1}, eps=0, precision={precision})",
            "step": "one Lloyd iteration; copy bytes per step = per-call bytes / iterations per call"}


def dense_job_line(E, X, C0, precision, steps, warmup):
    """Device-resident Lloyd steps of one job (rows, centers, assignments stay in HBM)."""
    mc = E.mc
    job = mc.Job(X, C0, msr=2, precision=precision, seed=7, ctx=E.ctx)
    job.assign()
    ms, launches, phases, clk = E.timed(job.lloyd_step, steps, warmup, profile=True)
    return job, ms, launches, phases, clk


def c3_tf32(args, E, X, C0, fp32_iters):
    """C3 in TF32: the same rows and kmeans++ centers as the BF16 headline."""
    n = X.shape[0]
    steps = max(3, min(args.steps, 10))
    job, ms, launches, phases, clk = dense_job_line(E, X, C0, "tf32", steps, max(args.warmup, 3))
    pk, pk_kind = peaks()
    out = {"metric": "Lloyd iters/s 4M x128 k=1024 (TF32 tensor-core assignment)", "value": 1000.0 / ms,
           "unit": "iters/s", "ms_per_step": ms, "steps": steps, "dtype": "tf32",
           "config": {"workload": f"dense {n}x{D}, {COMPONENTS} components, SQRL2, k={K}, kmeans++ centers "
                                  f"(the headline's), Lloyd iteration", "precision": "tf32"},
           "speedup_vs_fp32_gpu": (1000.0 / ms / fp32_iters) if fp32_iters else None,
           "recheck_rows_last_pass": job.recheck_count(),
           "accuracy_vs_fp64": fp64_objective_check(job, X, n),
           "roofline": tc_roofline(phases, n, "tf32", pk, pk_kind), "phases_ms_timed_region": phases,
           "gpu_launches": int(launches * steps), "clocks": clk}
    job.close()
    E.free()
    out["e2e"] = None if args.no_e2e else dense_e2e(E, X, C0, "tf32", 1)
    return out


# ------------------------------------------------------------------------------------
# C1: dense 10,000 x 50, k = 25, kmeans++ then 20 Lloyd updates, whole calls from host
# ------------------------------------------------------------------------------------
def c1_small(args):
    import torch
    import minicore_gb300 as mc
    X = make_small_data(0)
    ids, _, _ = mc.kmeanspp(X, 25, msr=2, seed=42)
    C0 = X[ids.astype(np.int64)]
    out, res = {}, {}
    steps = max(args.steps, 5)
    modes = {"graph": mc.LOOP_GRAPH, "fused": mc.LOOP_FUSED, "host": mc.LOOP_HOST}
    clk = Clocks().start()
    for name, mode in modes.items():
        mc.loop_mode(mode)
        for _ in range(max(args.warmup, 3)):
            mc.hcluster(X, C0, msr=2, eps=0.0, maxiter=19, seed=3)
        torch.cuda.synchronize()
        l0 = mc.kernel_launches()
        t = []
        for _ in range(steps):
            t0 = time.perf_counter()
            r = mc.hcluster(X, C0, msr=2, eps=0.0, maxiter=19, seed=3)
            t.append((time.perf_counter() - t0) * 1e3)
        res[name] = r
        t = np.sort(np.array(t))
        out[name] = {"ms_per_call_p50": float(np.percentile(t, 50)), "ms_per_call_min": float(t[0]),
                     "updates": int(r["numiter"]), "launches_per_call": (mc.kernel_launches() - l0) / steps}
    clocks = clk.stop()
    mc.loop_mode(mc.LOOP_AUTO)
    same = all(np.array_equal(res[m][key], res["host"][key]) and res[m]["finalcost"] == res["host"]["finalcost"]
               for m in ("graph", "fused") for key in ("asn", "costs", "centers"))
    best = min(out, key=lambda m: out[m]["ms_per_call_p50"])
    g = out[best]
    r = res[best]
    acc = fp64_sqrl2_check(X, r["centers"], r["asn"], r["costs"].astype(np.float64))
    acc["finalcost_gpu"] = r["finalcost"]
    acc["finalcost_rel_err_vs_fp64"] = abs(r["finalcost"] - acc["objective_fp64"]) / acc["objective_fp64"]
    cpu = None
    if not args.no_cpu:
        import oracle
        tt = []
        for _ in range(5):
            t0 = time.perf_counter()
            oracle.hcluster(X, C0, 2, 0.0, eps=0.0, maxiter=19, seed=3)
            tt.append(time.perf_counter() - t0)
        cpu = {"value": 1.0 / float(np.median(tt)), "unit": "calls/s", "cores": os.cpu_count() or 1,
               "kind": "port", "sample": "the whole oracle hcluster (20 updates) on the same 10000 x 50 rows and "
                                         "seeds, median of 5"}
    per_call = g["ms_per_call_p50"] * 1e-3
    return {"metric": "hcluster calls/s 10000x50 k=25 (20 updates, host arrays in and out)",
            "value": 1.0 / per_call, "unit": "calls/s", "loop_mode": best,
            "lloyd_iters_per_s": g["updates"] / per_call, "modes": out, "identical_across_modes": bool(same),
            "steps": steps, "dtype": "f32",
            "config": {"workload": "10000x50, 25 components U[-10,10]^50 sigma 1, k=25, kmeans++ seeds, "
                                   "maxiter=19 (20 updates), eps=0"},
            "roofline": {"bound": "launch latency", "achieved": g["launches_per_call"] / per_call,
                         "unit": "kernel launches/s", "peak": None, "frac": None, "traffic": None,
                         "note": f"{g['launches_per_call']:.0f} launches of a few microseconds per call; "
                                 "rows (2 MB) and centers sit in L2"},
            "accuracy_vs_fp64": acc, "cpu_baseline": cpu, "gpu_launches": int(g["launches_per_call"] * steps),
            "clocks": clocks,
            "e2e": {"value": 1.0 / per_call, "unit": "calls/s", "h2d_bytes_per_step": int(X.nbytes + C0.nbytes),
                    "d2h_bytes_per_step": int(C0.nbytes + X.shape[0] * (4 + 4)),
                    "call": "minicore_gb300.hcluster(host numpy rows and centers, maxiter=19, eps=0)"}}


# ------------------------------------------------------------------------------------
# C2: CSR 1M x 20,000, ~1500 nonzeros per row, MKL and JSD (prior 1), k = 50
# ------------------------------------------------------------------------------------
class CsrData:
    def __init__(self, n, seed=0):
        import torch
        self.n, self.d = n, CSR_D
        self.vals, self.idx, self.indptr = make_csr_counts(n, CSR_D, seed=seed)
        torch.cuda.synchronize()
        self.nnz = int(self.vals.numel())
        self.ipc = self.indptr.cpu()

    def device_matrix(self, mc):
        return mc.CSparseMatrix(data=self.vals, indices=self.idx, indptr=self.indptr, shape=(self.n, self.d))

    def sample(self, S):
        import scipy.sparse as sp
        ip = self.ipc[:S + 1].numpy().astype(np.int64)
        e = int(ip[-1])
        return sp.csr_matrix((self.vals[:e].cpu().numpy(), self.idx[:e].cpu().numpy().astype(np.int64), ip),
                             shape=(S, self.d))

    def centers_from_ids(self, ids):
        import torch
        C = torch.zeros((len(ids), self.d), dtype=torch.float32, device="cuda")
        for c, r in enumerate(ids):
            b, e = int(self.ipc[r]), int(self.ipc[r + 1])
            C[c, self.idx[b:e].long()] = self.vals[b:e]
        return C


def c2_csr(args, E, data, msr):
    """Sparse count workload, MKL (5) or JSD (4), prior 1, k = 50: D^2 seeding, then Lloyd
    iterations with rows resident in HBM.  The roofline is that of the assignment kernel:
    MKL against HBM (bytes), JSD against the measured logf rate (two logf per nonzero and
    center)."""
    import torch
    mc, _lib, lib = E.mc, E._lib, E.lib
    n, d, k, prior = data.n, data.d, CSR_K, 1.0
    name = {5: "MKL", 4: "JSD"}[msr]
    A = data.device_matrix(mc)
    M = mc._MatrixArg(A)
    u = torch.from_numpy(mc.uniforms(99, k)).cuda()
    ids = torch.empty(k, dtype=torch.int32, device="cuda")
    asn = torch.empty(n, dtype=torch.int32, device="cuda")
    costs = torch.empty(n, dtype=torch.float64, device="cuda")

    def seed():
        _lib.check(lib.mc_kmeanspp(E.ctx.handle, M.ref, k, msr, prior, None, mc._p(u), mc._p(ids), mc._p(asn),
                                   mc._p(costs)))
    kmpp_ms, _, _, _ = E.timed(seed, 1, 1)
    id_list = ids.cpu().tolist()
    C = data.centers_from_ids(id_list)
    del asn, costs
    job = mc.Job(A, C, msr=msr, prior=prior, ctx=E.ctx)
    job.assign()
    steps = max(3, min(args.steps, 10 if msr == 5 else 5))
    ms, launches, phases, clk = E.timed(job.lloyd_step, steps, max(args.warmup, 2) if msr == 5 else 2, profile=True)
    kms, kl = kernel_ms(phases, "assign_csr_sparse", "assign_csr_tiled")
    pk, pk_kind = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    algo_bytes = data.nnz * 8 + (n + 1) * 8 + n * 8 + n * 12 + k * d * 4
    if msr == 5:
        ach = algo_bytes / (kms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": None, "peak_source": f"{pk_kind} hbm_gbs",
                "kernel": "k_assign_sparse_pair<MKL> (sparse dot over each row's nonzeros, all centers)",
                "kernel_ms_per_launch": kms, "launches": kl,
                "algorithmic": f"nnz*8 + (n+1)*8 + n*20 + k*d*4 = {algo_bytes:.4g} bytes per launch"}
    else:
        rate = ctypes.c_double()
        _lib.check(lib.mc_diag_logf_rate(0, ctypes.byref(rate)))
        logs = 2.0 * data.nnz * k
        ach = logs / (kms * 1e-3)
        roof = {"bound": "logf (FP32 pipe)", "achieved": ach / 1e12, "peak": rate.value / 1e12, "unit": "Tlogf/s",
                "frac": ach / rate.value, "traffic": None,
                "peak_source": "measured: mc_diag_logf_rate (independent logf chains, full occupancy)",
                "kernel": "k_assign_sparse<JSD> (row groups by zero-entry value + sparse dot)",
                "kernel_ms_per_launch": kms, "launches": kl,
                "algorithmic": f"2*nnz*k = {logs:.4g} logf per launch",
                "hbm_frac_for_reference": algo_bytes / (kms * 1e-3) / 1e9 / hbm}
    # accuracy: the GPU's final assignment of a row sample against the oracle (the
    # reference's FP32 arithmetic) and against FP64
    Ch = np.empty((k, d), np.float32)
    asn_h = np.empty(n, np.uint32)
    cost_h = np.empty(n, np.float64)
    job.read(Ch, asn_h, cost_h)
    job.close()
    E.free()
    S = 20_000 if msr == 5 else 8_000
    sub = data.sample(S)
    acc = cpu = None
    if not args.no_cpu:
        import oracle
        oracle.build()
        t0 = time.perf_counter()
        oasn, ocost = oracle.assign(sub, Ch, msr, prior)
        t_assign = time.perf_counter() - t0
        acc = csr_accuracy(msr, sub, Ch, asn_h[:S], cost_h[:S], oasn, ocost, 2000 if msr == 5 else 200)
        t0 = time.perf_counter()
        oracle.hcluster(sub, Ch, msr, prior, eps=0.0, maxiter=0, seed=1)   # assign, update, assign
        t_iter = (time.perf_counter() - t0) - t_assign
        cpu = {"value": 1.0 / (t_iter * n / S), "unit": "iters/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"oracle Lloyd iteration (union-walk assignment + CSR centroid update) of the first {S} "
                         f"rows against the same {k} centers, scaled by {n}/{S}",
               "assign_passes_per_s": 1.0 / (t_assign * n / S)}
    e2e = None
    if not args.no_e2e:
        vh, ih, ph = pinned_copy(data.vals), pinned_copy(data.idx), pinned_copy(data.indptr)
        Ah = mc.CSparseMatrix(data=vh, indices=ih, indptr=ph, shape=(n, d))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ids_e, _, _ = mc.kmeanspp(Ah, k, msr=msr, prior=prior, seed=99, ctx=E.ctx)
        t_seed = time.perf_counter() - t0
        t0 = time.perf_counter()
        r = mc.hcluster(Ah, ids_e.astype(np.int64), msr=msr, prior=prior, eps=0.0, maxiter=E2E_ITERS - 1,
                        ctx=E.ctx)
        t_run = time.perf_counter() - t0
        it = int(r["numiter"])
        h2d = data.nnz * 8 + (n + 1) * 8
        e2e = {"value": it / t_run, "unit": "iters/s", "h2d_bytes_per_step": int(h2d / max(it, 1)),
               "d2h_bytes_per_step": int((k * d * 4 + n * 12) / max(it, 1)), "h2d_bytes_per_call": int(h2d),
               "iters_per_call": it, "kmeanspp_s_from_host": t_seed,
               "same_seeds_as_device_run": bool(np.array_equal(ids_e.astype(np.int64), np.array(id_list))),
               "call": f"minicore_gb300.hcluster(pinned host CSR, kmeans++ row ids, msr={msr}, prior=1, "
                       f"maxiter={E2E_ITERS - 1}, eps=0)",
               "step": "one Lloyd iteration; copy bytes per step = per-call bytes / iterations per call"}
        del vh, ih, ph, Ah
    tuned = {key: v for key, v in mc.autotune_report().get("entries", {}).items()
             if key.startswith(f"csr_sparse|msr{msr}|")}
    return {"metric": f"CSR {name} Lloyd iters/s 1Mx20000 k=50 (rows resident)", "value": 1000.0 / ms,
            "autotune_variants_ms": tuned,
            "unit": "iters/s", "ms_per_step": ms, "steps": steps, "dtype": "f32",
            "assign_ms_per_pass": kms, "kmeanspp_ms": kmpp_ms,
            "config": {"workload": f"CSR {n}x{d}, {CSR_NNZ_ROW} nnz/row Zipf(1.1) columns, NB(3,0.5) counts, "
                                   f"msr={msr} ({name}), prior=1, k={k}, kmeans++ centers, Lloyd iteration",
                       "l2": "rows 12 GB > L2"},
            "roofline": roof, "phases_ms_timed_region": phases, "accuracy": acc, "cpu_baseline": cpu,
            "gpu_launches": int(launches * steps), "clocks": clk, "e2e": e2e}


# ------------------------------------------------------------------------------------
# C4: coreset pipeline on 2M x 64
# ------------------------------------------------------------------------------------
def c4_coreset(args, E):
    """kmeans++ (k=100) -> LBK sensitivities + alias table -> 50,000 weighted draws ->
    weighted Lloyd on the coreset -> full-data objective of the coreset centers, against
    the objective of Lloyd on the full data from the same seeds.  Rows stay in HBM; every
    stage is timed with CUDA events on the library's stream."""
    torch, mc, _lib, lib = E.torch, E.mc, E._lib, E.lib
    n, d, k, m = args.coreset_rows, 64, 100, 50_000
    X = make_coreset_data(n, d)
    M = mc._MatrixArg(X)
    u = torch.from_numpy(mc.uniforms(77, k)).cuda()
    ids = torch.empty(k, dtype=torch.int32, device="cuda")
    asn = torch.empty(n, dtype=torch.int32, device="cuda")
    costs = torch.empty(n, dtype=torch.float64, device="cuda")
    cw = torch.empty(m, dtype=torch.float32, device="cuda")
    cidx = torch.empty(m, dtype=torch.int64, device="cuda")
    precision = "bf16"
    keep = {}

    def pipeline():
        t = [E.event()]
        _lib.check(lib.mc_kmeanspp(E.ctx.handle, M.ref, k, 2, 0.0, None, mc._p(u), mc._p(ids), mc._p(asn),
                                   mc._p(costs)))
        t.append(E.event())
        h = ctypes.c_void_p()
        _lib.check(lib.mc_sampler_create(E.ctx.handle, n, k, k, mc._p(costs), 1, mc._p(asn), None, 4, 0.0,
                                         ctypes.byref(h)))
        t.append(E.event())
        _lib.check(lib.mc_sampler_sample(h, m, 1234, 0, mc._p(cw), mc._p(cidx)))
        t.append(E.event())
        lib.mc_sampler_destroy(h)
        Xc = X[cidx].contiguous()
        C0 = X[ids.long()].contiguous()
        jc = mc.Job(Xc, C0, msr=2, weights=cw.double(), precision="fp32", seed=9, ctx=E.ctx)
        jc.run(eps=1e-4, maxiter=20)
        Cc = torch.empty((k, d), dtype=torch.float32, device="cuda")
        jc.read(Cc, None, None)
        t.append(E.event())
        jf = mc.Job(X, Cc, msr=2, precision=precision, seed=9, ctx=E.ctx)
        jf.assign()
        keep["obj"] = jf.cost()
        t.append(E.event())
        jc.close()
        keep["jf"], keep["C0"], keep["Cc"] = jf, C0, Cc
        return t

    for _ in range(max(args.warmup, 1)):
        pipeline()
        keep["jf"].close()
    torch.cuda.synchronize()
    clk = Clocks().start()
    l0 = lib.mc_kernel_launches()
    stage_ms = []
    steps = max(3, min(args.steps, 10))
    for s in range(steps):
        t = pipeline()
        torch.cuda.synchronize()
        stage_ms.append([t[i].elapsed_time(t[i + 1]) for i in range(len(t) - 1)])
        if s + 1 < steps:
            keep["jf"].close()
    launches = int(lib.mc_kernel_launches() - l0)
    clocks = clk.stop()
    stage = np.mean(np.array(stage_ms), axis=0)
    names = ["kmeanspp", "sensitivity_alias", "sample", "coreset_lloyd", "full_data_assign"]
    total_ms = float(stage.sum())
    acc = fp64_objective_check(keep["jf"], X, n)
    keep["jf"].close()
    jfull = mc.Job(X, keep["C0"], msr=2, precision=precision, seed=9, ctx=E.ctx)
    jfull.run(eps=1e-4, maxiter=20)
    obj_full = jfull.cost()
    jfull.close()
    pk, pk_kind = peaks()
    kmpp_bytes = k * n * d * 4 + k * n * 8 * 2
    achieved = kmpp_bytes / (stage[0] * 1e-3) / 1e9
    hbm = pk.get("hbm_gbs", 6800.0)
    cpu = None
    if not args.no_cpu:
        import oracle
        oracle.build()
        S = 200_000
        Xs = X[:S].cpu().numpy()
        tt = []
        for _ in range(3):
            t0 = time.perf_counter()
            oracle.kmeanspp(Xs, k, 2, 0.0, mc.uniforms(77, k))
            tt.append(time.perf_counter() - t0)
        per = float(np.median(tt)) * (n / S)
        cpu = {"value": 1.0 / per, "unit": "kmeans++ runs/s (k=100, 2M x 64)", "cores": os.cpu_count() or 1,
               "kind": "port", "sample": f"oracle kmeans++ on {S} rows, k={k}, median of 3, scaled by {n}/{S}",
               "gpu_kmeanspp_runs_per_s": 1000.0 / float(stage[0])}
    e2e = None
    if not args.no_e2e:
        Xh = pinned_copy(X)
        t0 = time.perf_counter()
        ids_e, asn_e, cost_e = mc.kmeanspp(Xh, k, msr=2, seed=77, ctx=E.ctx)
        cs = mc.CoresetSampler(ctx=E.ctx)
        cs.make_sampler(k, cost_e.astype(np.float64), asn_e.astype(np.uint32), seed=13, sens=4)
        wts, idx = cs.sample(m, seed=1234)
        Xn = Xh.numpy()
        Xc = np.ascontiguousarray(Xn[idx.astype(np.int64)])
        r = mc.hcluster(Xc, np.ascontiguousarray(Xn[ids_e.astype(np.int64)]), msr=2, weights=wts.astype(np.float64),
                        eps=1e-4, maxiter=20, seed=9, ctx=E.ctx)
        jf = mc.Job(Xh, r["centers"], msr=2, precision=precision, seed=9, ctx=E.ctx)
        jf.assign()
        obj_e = jf.cost()
        jf.close()
        t_e = time.perf_counter() - t0
        e2e = {"value": 1.0 / t_e, "unit": "pipelines/s", "h2d_bytes_per_step": int(2 * n * d * 4 + m * d * 4),
               "d2h_bytes_per_step": int(n * 12 + m * 12 + k * d * 4),
               "call": "minicore_gb300.kmeanspp -> CoresetSampler.make_sampler(sens=LBK)/sample -> hcluster("
                       "weighted coreset) -> Job(full rows).assign/cost, all from pinned host rows",
               "objective_coreset_centers_on_full_data": obj_e}
        del Xh
    E.free()
    return {"metric": "coreset pipelines/s 2M x 64 (kmeans++ k=100 -> LBK -> 50k draws -> weighted Lloyd)",
            "value": 1000.0 / total_ms, "unit": "pipelines/s", "ms_per_step": total_ms, "steps": steps,
            "dtype": "f32 (bf16 full-data assignment)",
            "config": {"workload": f"dense {n}x{d}, 200 components N(0,4I) means, Dirichlet(0.3) weights; "
                                   f"kmeans++ k={k}; LBK sensitivities; alias; m={m}; weighted Lloyd eps 1e-4 "
                                   f"<= 20 updates", "l2": "rows 512 MB > L2"},
            "stages_ms": dict(zip(names, map(float, stage))),
            "objective": {"coreset_centers_on_full_data": keep["obj"], "full_data_lloyd": obj_full,
                          "ratio": keep["obj"] / obj_full},
            "accuracy_vs_fp64": acc,
            "roofline": {"bound": "hbm", "kernel": "kmeans++ (k passes over the rows)", "achieved": achieved,
                         "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                         "peak_source": f"{pk_kind} hbm_gbs",
                         "algorithmic": f"k*n*d*4 + 2*k*n*8 = {kmpp_bytes:.4g} bytes"},
            "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clocks, "e2e": e2e}


# ------------------------------------------------------------------------------------
# the reference arm: the oracle's CPU Lloyd iteration on the headline workload
# ------------------------------------------------------------------------------------
def reference_arm(args):
    """--impl reference: the oracle's CPU Lloyd iteration (one assignment + one centroid
    update, FT = float), all host threads, on a sample of the 4M x 128 mixture, scaled to
    the full row count; W warm-up iterations, then the median of K."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle
    oracle.build()
    rng = np.random.default_rng(0)
    S = args.cpu_sample
    mu = rng.normal(size=(COMPONENTS, D)) * 2.0
    Xs = (mu[rng.integers(0, COMPONENTS, S)] + rng.normal(size=(S, D))).astype(np.float32)
    C = Xs[rng.choice(S, K, replace=False)]
    for _ in range(args.warmup):
        oracle.hcluster(Xs, C, 2, 0.0, eps=0.0, maxiter=0, seed=1)
    times = []
    for _ in range(max(args.steps, 1)):
        t_iter, _ = cpu_lloyd_iteration(Xs, C, repeats=1)
        times.append(t_iter)
    per_iter_full = float(np.median(times)) * (args.n / S)
    v = 1.0 / per_iter_full
    spread = (max(times) - min(times)) / float(np.median(times))
    line = {"metric": "Lloyd iters/s 4M x128 k=1024", "value": v, "unit": "iters/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_iter_full * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"dense {args.n}x{D} gaussian mixture, SQRL2, k={K}, Lloyd iteration",
                       "sample_rows": S},
            "cpu_baseline": {"value": v, "unit": "iters/s", "cores": threads, "kind": "port",
                             "sample": f"{S} rows x k={K}: one assignment + one centroid update of the oracle per "
                                       f"iteration (median of {len(times)}, spread {spread:.2%}), scaled by "
                                       f"{args.n}/{S}"},
            "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------------------------------
# the default line
# ------------------------------------------------------------------------------------
def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "serving":
        return serving_main(args)
    if args.workload == "coreset":
        E = Env(0)
        print(json.dumps(c4_coreset(args, E)))
        return
    if args.workload in ("pcmp", "minibatch", "soft", "coreset_mb"):
        return next_rows_bench(args)
    if args.workload == "small":
        Env(0)
        print(json.dumps(c1_small(args)))
        return
    if args.workload in ("csr_mkl", "csr_jsd"):
        E = Env(0)
        data = CsrData(args.csr_rows)
        print(json.dumps(c2_csr(args, E, data, 5 if args.workload == "csr_mkl" else 4)))
        return
    if args.workload == "csr_l1":
        return csr_l1_bench(args)
    if args.workload == "tf32":
        args.precision = "tf32"
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    E = Env(local)
    mc, _lib, lib = E.mc, E._lib, E.lib
    n = args.n
    X = make_data(n, seed=rank)
    # kmeans++ centers (untimed setup)
    M = mc._MatrixArg(X)
    u = torch.from_numpy(mc.uniforms(1234, K)).cuda()
    idst = torch.empty(K, dtype=torch.int32, device="cuda")
    asn0 = torch.empty(n, dtype=torch.int32, device="cuda")
    costs0 = torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.check(lib.mc_kmeanspp(E.ctx.handle, M.ref, K, 2, 0.0, None, mc._p(u), mc._p(idst), mc._p(asn0),
                               mc._p(costs0)))
    torch.cuda.synchronize()
    C0 = X[idst.long()].contiguous()
    del asn0, costs0

    job = mc.Job(X, C0, msr=2, precision=args.precision, seed=7, ctx=E.ctx)
    job.assign()
    for _ in range(args.warmup):
        job.lloyd_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = Clocks().start()
    torch.cuda.synchronize()
    lib.mc_profile_reset()
    lib.mc_profile_enable(1)  # CUDA events around the library's phases, on this stream
    l0 = lib.mc_kernel_launches()
    torch.cuda.nvtx.range_push("lloyd_timed")
    ev0 = E.event()
    for _ in range(args.steps):
        job.lloyd_step()
    ev1 = E.event()
    torch.cuda.nvtx.range_pop()
    launches = int(lib.mc_kernel_launches() - l0)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    lib.mc_profile_enable(0)
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.check(lib.mc_profile_report(buf, len(buf)))
    phases = json.loads(buf.value.decode())
    ms_per_step, value = replica_throughput(ev0.elapsed_time(ev1), args.steps, world, "cuda")
    recheck = job.recheck_count()
    accuracy = fp64_objective_check(job, X, n) if rank == 0 else None
    pk, pk_kind = peaks()
    if args.precision == "fp32":
        kms, kl = kernel_ms(phases, "assign_dense_fp32")
        flops = 2.0 * n * K * D
        roofline = {"bound": "fp32", "achieved": flops / (kms * 1e-3) / 1e12, "peak": None, "unit": "TFLOP/s",
                    "frac": None, "traffic": None, "kernel": "k_assign_tiled<SQRL2>", "kernel_ms_per_launch": kms,
                    "launches": kl}
    else:
        roofline = tc_roofline(phases, n, args.precision, pk, pk_kind)
    job.close()
    E.free()

    # the plain FP32 GPU kernel on the same iteration (the comparison the metric names)
    fp32 = None
    if args.precision != "fp32":
        j32 = mc.Job(X, C0, msr=2, precision="fp32", seed=7, ctx=E.ctx)
        j32.assign()
        ms32, _, _, _ = E.timed(j32.lloyd_step, 2, 1)
        fp32 = 1000.0 / ms32
        j32.close()
        E.free()

    e2e = None if args.no_e2e else dense_e2e(E, X, C0, args.precision, max(1, min(args.steps, 3)))
    E.free()

    configs = {}
    if rank == 0 and not args.no_configs and args.workload == "dense" and n == N:
        configs["C3_tf32"] = _guard(lambda: c3_tf32(args, E, X, C0, fp32))
    del X
    E.free()

    cpu = None
    if not args.no_cpu and rank == 0:
        ref = cpu_reference_line(steps=5, warmup=1, sample=args.cpu_sample)
        if ref:
            cpu = dict(ref["cpu_baseline"])
        if isinstance(configs.get("C3_tf32"), dict) and "error" not in configs["C3_tf32"]:
            configs["C3_tf32"]["cpu_baseline"] = cpu  # the same CPU Lloyd iteration (the oracle is FP32)

    if rank == 0 and not args.no_configs and args.workload == "dense":
        configs["C1_small"] = _guard(lambda: c1_small(args))
        E.free()
        data = _guard(lambda: CsrData(args.csr_rows))
        if isinstance(data, CsrData):
            configs["C2_csr_mkl"] = _guard(lambda: c2_csr(args, E, data, 5))
            configs["C2_csr_jsd"] = _guard(lambda: c2_csr(args, E, data, 4))
        del data
        E.free()
        configs["C4_coreset"] = _guard(lambda: c4_coreset(args, E))
        E.free()

    serving = None
    if not args.no_serving and rank == 0:
        serving = serving_bench(1000, rate=200.0, slots=args.slots, saturation_jobs=250)

    if rank == 0:
        line = {"metric": "Lloyd iters/s 4M x128 k=1024", "value": value, "unit": "iters/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": args.precision, "data": "synthetic",
                "config": {"workload": f"dense {n}x{D} gaussian mixture ({COMPONENTS} comps), SQRL2, k={K}, "
                                       f"kmeans++ centers, Lloyd iteration",
                           "precision": args.precision, "parallelism": f"replicas{world}",
                           "l2": "inputs (2 GiB f32) larger than L2; no flush"},
                "fp32_gpu_iters_per_s": fp32,
                "speedup_vs_fp32_gpu": (value / world / fp32) if fp32 else None,
                "recheck_rows_last_pass": recheck,
                "accuracy_vs_fp64": accuracy,
                "roofline": roofline, "phases_ms_timed_region": phases,
                "autotune_tc": tc_autotune_entries(args.precision),
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk,
                "job_latency_ms": (serving or {}).get("latency_ms"),
                "serving": serving,
                "configs": configs}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def _guard(fn):
    """A sub-line that fails reports its error instead of ending the run."""
    try:
        return fn()
    except Exception as e:  # noqa: BLE001
        import traceback
        traceback.print_exc()
        return {"error": f"{type(e).__name__}: {e}"}


if __name__ == "__main__":
    main()
