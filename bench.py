#!/usr/bin/env python3
"""Benchmark: Lloyd iterations/s on the dense 4M x 128, k=1024 Gaussian-mixture workload.

A step is one Lloyd iteration (centroid update + hard assignment) over all rows.

* value: device-resident rows/centers (torch tensors handed to the C ABI), K steps timed
  with CUDA events on the library's stream, barrier + synchronize on both sides.  The rows
  (2 GiB f32 + 1 GiB bf16 copy) exceed the 129 MB L2, so no flush is needed between steps.
* e2e: the reference-facing call (mc_hcluster through minicore_gb300.hcluster) with host
  buffers in pinned memory: each step uploads the rows, runs kmeans++-seeded centers
  through 10 Lloyd updates and reads back centers / assignments / costs.
* roofline: the assignment kernel (the dominant launch), timed alone with CUDA events.
* cpu_baseline / --impl reference: the oracle (C++/OpenMP restatement of the reference's
  CPU path) on a row sample, scaled to the full row count.
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16", choices=["bf16", "tf32", "fp32"])
    ap.add_argument("--n", type=int, default=N)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="dense", choices=["dense", "csr_mkl", "csr_jsd", "csr_l1", "serving", "coreset", "pcmp",
                                                         "minibatch", "soft", "small", "coreset_mb"],
                    help="dense: the 4M x 128 k=1024 Lloyd workload (the default line); csr_*: the sparse "
                         "count-data workload (1M x 20000, 1500 nnz/row, k=50) assignment pass; serving: "
                         "the Poisson job stream through the continuous-batching server; coreset: the "
                         "2M x 64 kmeans++ -> sensitivity -> sampling -> weighted Lloyd pipeline")
    ap.add_argument("--coreset-rows", type=int, default=2_000_000)
    ap.add_argument("--serving-jobs", type=int, default=4000,
                    help="jobs in the --workload serving stream (the full stream is 20000)")
    ap.add_argument("--serving-rate", type=float, default=200.0)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the short serving run (p50/p99 job latency) in the default line")
    ap.add_argument("--csr-rows", type=int, default=1_000_000)
    return ap.parse_args()


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def make_data(n, seed=0):
    """1024 component means ~N(0, 4I), points ~N(mean, I) (seeded, generated on the GPU)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    mu = torch.randn(COMPONENTS, D, generator=g, device="cuda") * 2.0
    lab = torch.randint(0, COMPONENTS, (n,), generator=g, device="cuda")
    X = torch.randn(n, D, generator=g, device="cuda")
    X.add_(mu[lab])
    return X.contiguous()


def make_csr_counts(n, d=20_000, nnz_row=1500, seed=0, chunk=4096):
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


def csr_bench(args):
    """Sparse count workload: D^2 seeding (k=50) then the timed assignment pass (MKL or JSD,
    prior 1) with rows resident in HBM; csr_l1: the timed step is one L1 Lloyd iteration
    (sparse coordinate-wise medians of the clusters, then the L1 assignment pass)."""
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
           "roofline": {"bound": "hbm" if msr == 5 else "compute", "achieved": algo_bytes / (kms * 1e-3) / 1e9,
                        "peak": pk.get("hbm_gbs", 6767.7), "unit": "GB/s",
                        "frac": algo_bytes / (kms * 1e-3) / 1e9 / pk.get("hbm_gbs", 6767.7),
                        "algorithmic_bytes": algo_bytes, "kernel_ms": kms, "peak_source": pk_kind},
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


def coreset_bench(args):
    """Coreset pipeline on 2M x 64 (200-component mixture, Dirichlet(0.3) component
    weights): kmeans++ (k=100) -> LBK sensitivities + alias table -> 50,000 weighted draws
    -> weighted Lloyd on the coreset -> full-data objective of the coreset centers, against
    the objective of Lloyd on the full data from the same seeds.  Rows stay in HBM; every
    stage is timed with CUDA events on the library's stream."""
    import torch
    import minicore_gb300 as mc
    from minicore_gb300 import _lib
    torch.cuda.set_device(0)
    lib = _lib.load()
    ctx = mc.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    n, d, k, m, comps = args.coreset_rows, 64, 100, 50_000, 200
    rng = np.random.default_rng(0)
    wts = torch.from_numpy(rng.dirichlet(np.full(comps, 0.3))).cuda()
    g = torch.Generator(device="cuda").manual_seed(0)
    mu = torch.randn(comps, d, generator=g, device="cuda") * 2.0
    lab = torch.multinomial(wts, n, replacement=True, generator=g)
    X = torch.randn(n, d, generator=g, device="cuda").add_(mu[lab]).contiguous()
    del lab
    M = mc._MatrixArg(X)
    u = torch.from_numpy(mc.uniforms(77, k)).cuda()
    ids = torch.empty(k, dtype=torch.int32, device="cuda")
    asn = torch.empty(n, dtype=torch.int32, device="cuda")
    costs = torch.empty(n, dtype=torch.float64, device="cuda")
    cw = torch.empty(m, dtype=torch.float32, device="cuda")
    cidx = torch.empty(m, dtype=torch.int64, device="cuda")
    precision = args.precision

    def ev():
        e = torch.cuda.Event(enable_timing=True)
        e.record(stream)
        return e

    def pipeline():
        t = [ev()]
        _lib.check(lib.mc_kmeanspp(ctx.handle, M.ref, k, 2, 0.0, None, mc._p(u), mc._p(ids), mc._p(asn),
                                   mc._p(costs)))
        t.append(ev())
        h = ctypes.c_void_p()
        _lib.check(lib.mc_sampler_create(ctx.handle, n, k, k, mc._p(costs), 1, mc._p(asn), None, 4, 0.0,
                                         ctypes.byref(h)))
        t.append(ev())
        _lib.check(lib.mc_sampler_sample(h, m, 1234, 0, mc._p(cw), mc._p(cidx)))
        t.append(ev())
        lib.mc_sampler_destroy(h)
        Xc = X[cidx].contiguous()
        C0 = X[ids.long()].contiguous()
        jc = mc.Job(Xc, C0, msr=2, weights=cw.double(), precision="fp32", seed=9, ctx=ctx)
        jc.run(eps=1e-4, maxiter=20)
        Cc = torch.empty((k, d), dtype=torch.float32, device="cuda")
        jc.read(Cc, None, None)
        t.append(ev())
        # the coreset centers on the full data: one assignment pass + FP64 objective
        jf = mc.Job(X, Cc, msr=2, precision=precision, seed=9, ctx=ctx)
        jf.assign()
        obj_core = jf.cost()
        t.append(ev())
        jc.close()
        jf.close()
        return t, obj_core, C0

    for _ in range(max(args.warmup, 1)):
        pipeline()
    torch.cuda.synchronize()
    clocks = Clocks()
    clocks.start()
    l0 = lib.mc_kernel_launches()
    stage_ms = []
    for _ in range(args.steps):
        t, obj_core, C0 = pipeline()
        torch.cuda.synchronize()
        stage_ms.append([t[i].elapsed_time(t[i + 1]) for i in range(len(t) - 1)])
    launches = int(lib.mc_kernel_launches() - l0)
    clk = clocks.stop()
    stage = np.mean(np.array(stage_ms), axis=0)
    names = ["kmeanspp", "sensitivity_alias", "sample", "coreset_lloyd", "full_data_assign"]
    total_ms = float(stage.sum())
    # the full-data solution from the same seeds, for the objective ratio (untimed)
    jfull = mc.Job(X, C0, msr=2, precision=precision, seed=9, ctx=ctx)
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
        S = 100_000
        Xs = X[:S].cpu().numpy()
        t0 = time.perf_counter()
        oracle.kmeanspp(Xs, k, 2, 0.0, mc.uniforms(77, k))
        per = (time.perf_counter() - t0) * (n / S)
        cpu = {"value": 1.0 / per, "unit": "kmeans++ runs/s (k=100, 2M x 64)", "cores": os.cpu_count() or 1,
               "kind": "port", "sample": f"oracle kmeans++ on {S} rows, k={k}, scaled by {n}/{S}"}
    line = {"metric": "coreset pipelines/s 2M x 64 (kmeans++ k=100 -> LBK -> 50k draws -> weighted Lloyd)",
            "value": 1000.0 / total_ms, "unit": "pipelines/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if precision == "fp32" else f"f32 ({precision} full-data assign)",
            "data": "synthetic",
            "config": {"workload": f"dense {n}x{d}, {comps} components N(0,4I) means, Dirichlet(0.3) weights; "
                                   f"kmeans++ k={k}; LBK sensitivities; alias; m={m}; weighted Lloyd eps 1e-4 "
                                   f"<= 20 updates", "l2": "rows 512 MB > L2"},
            "stages_ms": dict(zip(names, map(float, stage))),
            "objective": {"coreset_centers_on_full_data": obj_core, "full_data_lloyd": obj_full,
                          "ratio": obj_core / obj_full},
            "roofline": {"bound": "hbm", "kernel": "kmeans++ (k passes over the rows)", "achieved": achieved,
                         "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                         "peak_source": f"{pk_kind} hbm_gbs",
                         "algorithmic": f"k*n*d*4 + 2*k*n*8 = {kmpp_bytes:.4g} bytes"},
            "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clk,
            "e2e": None}
    print(json.dumps(line))


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


def make_serving_pool(seed=0):
    """Device-resident row pools the serving jobs slice: per d in {32, 64, 128, 512}, a dense
    200-component Gaussian mixture (means ~N(0, 4I), sigma 1) and a CSR count matrix at 1%
    density (Bernoulli(0.01) columns, every row at least one entry, NB counts), 200k rows."""
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
        else:
            v, c, ip = csr[d]
            b, e = int(ip[off]), int(ip[off + n])
            X = mc.CSparseMatrix(data=v[b:e], indices=c[b:e], indptr=(ip[off:off + n + 1] - b).contiguous(),
                                 shape=(n, d))
            spec = dict(matrix=X, k=k, msr=5, prior=1.0, precision="fp32")
            kind = "csr_mkl"
        spec.update(eps=1e-4, maxiter=10, seed=1000 + i)
        jobs.append({"spec": spec, "t": float(arrivals[i]), "n": n, "d": d, "k": k, "kind": kind})
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


def serving_bench(njobs, rate=200.0, slots=8, seed=0, saturation_jobs=None, serial=False):
    """The serving form: a seeded Poisson stream of uneven jobs through mc_server (continuous
    batching over `slots` concurrent slots, admission by free device memory)."""
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
    with mc.Server(slots=slots) as srv:
        run_serving(srv, warm, open_loop=False)
        srv.reset_stats()
        clocks = Clocks()
        clocks.start()
        l0 = lib.mc_kernel_launches()
        res, wall = run_serving(srv, jobs, open_loop=True)
        launches = int(lib.mc_kernel_launches() - l0)
        clk = clocks.stop()
        st = srv.stats()
        srv.reset_stats()
        res_s, wall_s = run_serving(srv, sat, open_loop=False)
        st_s = srv.stats()
    tot = np.array([r["total_ms"] for r in res])
    run = np.array([r["run_ms"] for r in res])
    qms = np.array([r["queue_ms"] for r in res])
    rows_iters = sum(j["n"] * (r["numiter"] + 1) for j, r in zip(jobs, res))
    d2h = sum(j["k"] * j["d"] * 4 + j["n"] * 12 for j in jobs)

    def pct(a):
        return {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99)), "mean": float(a.mean())}

    by_kind = {}
    for kind in ("dense_sqrl2_bf16", "csr_mkl"):
        sel = np.array([j["kind"] == kind for j in jobs])
        if sel.any():
            by_kind[kind] = {"jobs": int(sel.sum()), "total_ms": pct(tot[sel])}
    out = {"jobs": njobs, "rate_per_s": rate, "slots": slots, "wall_s": wall, "jobs_per_s": njobs / wall,
           "latency_ms": {"total": pct(tot), "queue": pct(qms), "run": pct(run)},
           "server_stats": st, "by_kind": by_kind, "row_iterations_per_s": rows_iters / wall,
           "gpu_launches": launches, "clocks": clk, "d2h_bytes": int(d2h),
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
    s = serving_bench(args.serving_jobs, rate=args.serving_rate, slots=args.slots, serial=True)
    line = {"metric": "serving jobs/s (Poisson 200/s mix of uneven clustering jobs); p50/p99 job latency",
            "value": s["jobs_per_s"], "unit": "jobs/s", "n_gpus": 1, "steps": s["jobs"], "warmup": 16,
            "ms_per_step": 1000.0 * s["wall_s"] / s["jobs"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 (dense SQRL2) / f32 (CSR MKL)", "data": "synthetic",
            "config": {"workload": f"{s['jobs']} jobs, Poisson {args.serving_rate}/s, n logU[1e3,2e5], "
                                   f"d in {{32,64,128,512}}, k logU[5,200], half dense SQRL2 BF16, half CSR "
                                   f"MKL 1% density; kmeans++ then Lloyd (eps 1e-4, 10 updates)",
                       "slots": args.slots, "l2": "row pools 0.6 GB dense + CSR, jobs slice them"},
            "latency_ms": s["latency_ms"], "serving": s, "gpu_launches": s["gpu_launches"],
            "clocks": s["clocks"],
            "e2e": {"value": s["jobs_per_s"], "unit": "jobs/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(s["d2h_bytes"] / s["jobs"]),
                    "call": "minicore_gb300.Server.submit/wait (rows resident, outputs to host)"}}
    print(json.dumps(line))


class Clocks:
    """nvidia-smi sampling during the timed region."""

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


def fp64_objective_check(job, X, n, sample=100_000, seed=5):
    """After the timed steps: the job's assignment and objective on a fixed row subsample
    against an FP64 computation (numpy, float64 GEMM form of the squared distances) with
    the same centers."""
    import torch
    k, d = job.k, X.shape[1]
    C = np.empty((k, d), np.float32)
    asn = np.empty(n, np.uint32)
    costs = np.empty(n, np.float64)
    job.read(C, asn, costs)
    S = np.sort(np.random.default_rng(seed).choice(n, min(sample, n), replace=False))
    Xs = X[torch.from_numpy(S).cuda()].cpu().numpy().astype(np.float64)
    C64 = C.astype(np.float64)
    cn = (C64 * C64).sum(1)
    best = np.empty(len(S))
    arg = np.empty(len(S), np.int64)
    for i in range(0, len(S), 8192):
        x = Xs[i:i + 8192]
        dist = (x * x).sum(1)[:, None] - 2.0 * (x @ C64.T) + cn[None, :]
        arg[i:i + 8192] = dist.argmin(1)
        best[i:i + 8192] = np.maximum(dist.min(1), 0.0)
    obj64 = float(best.sum())
    obj_gpu = float(costs[S].sum())
    # the FP64 distance to the center the GPU picked, where the argmins differ
    diff = np.nonzero(arg != asn[S])[0]
    gap = 0.0
    if len(diff):
        xd = Xs[diff]
        cd = C64[asn[S][diff].astype(np.int64)]
        gap = float((((xd - cd) ** 2).sum(1) - best[diff]).max())
    return {"sample_rows": int(len(S)), "objective_gpu": obj_gpu, "objective_fp64": obj64,
            "rel_err": abs(obj_gpu - obj64) / obj64, "argmin_agreement": float(1.0 - len(diff) / len(S)),
            "max_fp64_gap_where_argmin_differs": gap}


def cpu_baseline(X_sample, C, threads):
    """One Lloyd iteration (assignment + centroid update) of the oracle on a row sample."""
    import oracle
    oracle.build()
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    t0 = time.perf_counter()
    oracle.hcluster(X_sample, C, 2, 0.0, eps=0.0, maxiter=0, seed=1)  # assign, update, assign
    t = time.perf_counter() - t0
    # two assignment passes + one centroid update; a Lloyd iteration is one of each
    per_iter = t / 2.0
    return per_iter


def reference_arm(args):
    """--impl reference: the oracle's CPU Lloyd iteration, all host threads, on a sample."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    rng = np.random.default_rng(0)
    S = 20_000
    mu = rng.normal(size=(COMPONENTS, D)) * 2.0
    Xs = (mu[rng.integers(0, COMPONENTS, S)] + rng.normal(size=(S, D))).astype(np.float32)
    C = Xs[rng.choice(S, K, replace=False)]
    for _ in range(args.warmup):
        pass
    times = []
    for _ in range(max(args.steps, 1)):
        times.append(cpu_baseline(Xs, C, threads))
    per_iter_full = float(np.mean(times)) * (args.n / S)
    v = 1.0 / per_iter_full
    line = {"metric": "Lloyd iters/s 4M x128 k=1024", "value": v, "unit": "iters/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_iter_full * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"dense {args.n}x{D} gaussian mixture, SQRL2, k={K}, Lloyd iteration",
                       "sample_rows": S},
            "cpu_baseline": {"value": v, "unit": "iters/s", "cores": threads, "kind": "port",
                             "sample": f"{S} rows x k={K} (one assignment + centroid update), scaled by {args.n}/{S}"},
            "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def small_bench(args):
    """The small reference configuration (10,000 x 50, 25 Gaussian components ~U[-10, 10]^50,
    unit variance): kmeans++ (k = 25) then hcluster(maxiter=19, eps=0), i.e. 20 updates, from
    host NumPy arrays through the public API.  Timed per whole call, with the Lloyd loop as one
    CUDA graph and as a host loop (identical results, checked)."""
    import time
    import torch
    import minicore_gb300 as mc
    rng = np.random.default_rng(0)
    mu = rng.uniform(-10, 10, (25, 50))
    X = (mu[rng.integers(0, 25, 10000)] + rng.normal(size=(10000, 50))).astype(np.float32)
    ids, _, _ = mc.kmeanspp(X, 25, msr=2, seed=42)
    C0 = X[ids.astype(np.int64)]
    out = {}
    res = {}
    modes = {"graph": mc.LOOP_GRAPH, "fused": mc.LOOP_FUSED, "host": mc.LOOP_HOST}
    for name, mode in modes.items():
        mc.loop_mode(mode)
        for _ in range(args.warmup):
            mc.hcluster(X, C0, msr=2, eps=0.0, maxiter=19, seed=3)
        torch.cuda.synchronize()
        l0 = mc.kernel_launches()
        t = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            r = mc.hcluster(X, C0, msr=2, eps=0.0, maxiter=19, seed=3)
            t.append((time.perf_counter() - t0) * 1e3)
        res[name] = r
        t = np.sort(np.array(t))
        out[name] = {"ms_per_call_p50": float(np.percentile(t, 50)), "ms_per_call_min": float(t[0]),
                     "updates": int(r["numiter"]), "launches_per_call": (mc.kernel_launches() - l0) / args.steps}
    mc.loop_mode(mc.LOOP_AUTO)
    same = all(np.array_equal(res[m][key], res["host"][key]) and res[m]["finalcost"] == res["host"]["finalcost"]
               for m in ("graph", "fused") for key in ("asn", "costs", "centers"))
    best = min(out, key=lambda m: out[m]["ms_per_call_p50"])
    g = out[best]
    cpu = None
    if not args.no_cpu:
        import oracle
        t0 = time.perf_counter()
        oracle.hcluster(X, C0, 2, 0.0, eps=0.0, maxiter=19, seed=3)
        cpu = {"value": 1.0 / (time.perf_counter() - t0), "unit": "calls/s", "cores": os.cpu_count() or 1,
               "kind": "port", "sample": "the whole oracle hcluster on the same 10000 x 50 rows and seeds"}
    print(json.dumps({"metric": "hcluster calls/s 10000x50 k=25 (20 updates, host arrays in and out)",
                      "value": 1000.0 / g["ms_per_call_p50"], "unit": "calls/s", "loop_mode": best,
                      "lloyd_iters_per_s": g["updates"] * 1000.0 / g["ms_per_call_p50"],
                      "modes": out, "identical": bool(same), "cpu_baseline": cpu,
                      "steps": args.steps, "warmup": args.warmup, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": "10000x50, 25 components, k=25, kmeans++ seeds, maxiter=19, eps=0"}}))


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "serving":
        return serving_main(args)
    if args.workload == "coreset":
        return coreset_bench(args)
    if args.workload in ("pcmp", "minibatch", "soft", "coreset_mb"):
        return next_rows_bench(args)
    if args.workload == "small":
        return small_bench(args)
    if args.workload != "dense":
        return csr_bench(args)
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    import minicore_gb300 as mc
    ctx = mc.Context(local)
    # a dedicated (non-default) stream: the library launches on it and the CUDA events
    # that time the steps are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    n = args.n
    X = make_data(n, seed=rank)
    # kmeans++ centers (untimed setup), ids on the host
    seeds = mc.uniforms(1234, K)
    ids = np.empty(K, np.uint32)
    asn0 = torch.empty(n, dtype=torch.int32, device="cuda")
    costs0 = torch.empty(n, dtype=torch.float64, device="cuda")
    from minicore_gb300 import _lib
    M = mc._MatrixArg(X)
    u = torch.from_numpy(seeds).cuda()
    idst = torch.empty(K, dtype=torch.int32, device="cuda")
    _lib.check(_lib.load().mc_kmeanspp(ctx.handle, M.ref, K, 2, 0.0, None, mc._p(u), mc._p(idst), mc._p(asn0),
                                       mc._p(costs0)))
    torch.cuda.synchronize()
    ids = idst.cpu().numpy().astype(np.int64)
    C0 = X[torch.from_numpy(ids).cuda()].contiguous()
    del asn0, costs0

    job = mc.Job(X, C0, msr=2, precision=args.precision, seed=7, ctx=ctx)
    job.assign()
    for _ in range(args.warmup):
        job.lloyd_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = Clocks()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    lib = _lib.load()
    lib.mc_profile_reset()
    lib.mc_profile_enable(1)  # CUDA events around the library's phases, on this stream
    l0 = lib.mc_kernel_launches()
    torch.cuda.nvtx.range_push("lloyd_timed")
    ev0.record(stream)
    for _ in range(args.steps):
        job.lloyd_step()
    ev1.record(stream)
    torch.cuda.nvtx.range_pop()
    launches = int(lib.mc_kernel_launches() - l0)
    torch.cuda.synchronize()
    clk = clocks.stop()
    lib.mc_profile_enable(0)
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.check(lib.mc_profile_report(buf, len(buf)))
    phases = json.loads(buf.value.decode())
    ms_per_step, value = replica_throughput(ev0.elapsed_time(ev1), args.steps, world, "cuda")
    recheck = job.recheck_count()
    accuracy = fp64_objective_check(job, X, n) if rank == 0 else None

    # dominant kernel: the tensor-core assignment kernel (two passes per assignment) or the
    # FP32 tiled kernel, from the events recorded over the timed region
    pk, pk_kind = peaks()
    flops = 2.0 * n * K * D
    if args.precision == "fp32":
        kname, kinfo = "assign_dense_fp32 (k_assign_tiled)", phases.get("assign_dense_fp32", {})
        launches_k = kinfo.get("count", 0)
        avg_ms = kinfo.get("ms", float("nan")) / max(launches_k, 1)
        peak, unit = None, "TFLOP/s"
    else:
        # pass 1 is the full GEMM (every row x every center); pass 2 runs over the rows
        # whose top-2 margin is inside the rounding bound only
        p1 = phases.get("tc_pass1_top2", {})
        launches_k = p1.get("count", 0)
        avg_ms = p1.get("ms", float("nan")) / max(launches_k, 1)
        kname = f"k_tc_assign<{args.precision}, TC_TOP2> (pass 1: every row x every center)"
        peak, unit = pk.get("bf16_tflops", 1935.7), "TFLOP/s"
    achieved = flops / (avg_ms * 1e-3) / 1e12
    traffic = None  # DRAM bytes per launch from the committed ncu summary (scaled to 4M rows)
    if args.precision == "bf16" and n == N:
        try:
            for line in open(os.path.join(ROOT, "profiles", "k_tc_assign_bf16_4Mx128_k1024.md")):
                if line.startswith("traffic_bytes_per_launch_scaled_to_4M:"):
                    traffic = float(line.split(":")[1].split()[0])
        except OSError:
            traffic = None
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": unit,
                "frac": (achieved / peak) if peak else None, "traffic": traffic,
                "peak_source": f"{pk_kind} bf16_tflops (burst)", "kernel": kname,
                "kernel_ms_per_launch": avg_ms, "launches": launches_k,
                "algorithmic": f"2*n*k*d = {flops:.4g} FLOP per launch (n={n}, k={K}, d={D})"}

    # FP32 plain kernel for the same iteration (the comparison named by the metric)
    fp32 = None
    if args.precision != "fp32":
        j32 = mc.Job(X, C0, msr=2, precision="fp32", seed=7, ctx=ctx)
        j32.assign()
        j32.lloyd_step()
        torch.cuda.synchronize()
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record(stream)
        for _ in range(2):
            j32.lloyd_step()
        b1.record(stream)
        torch.cuda.synchronize()
        fp32 = 1000.0 / (b0.elapsed_time(b1) / 2)
        j32.close()

    # e2e: hcluster from pinned host buffers, 10 Lloyd updates per step
    e2e = None
    if not args.no_e2e:
        Xh = torch.empty((n, D), dtype=torch.float32, pin_memory=True)
        Xh.copy_(X)
        Ch = C0.cpu().numpy()
        Xn = Xh.numpy()
        mc.hcluster(Xn, Ch, msr=2, eps=0.0, maxiter=1, precision=args.precision, ctx=ctx)  # warm
        torch.cuda.synchronize()
        e_steps = max(1, min(args.steps, 3))
        t0 = time.perf_counter()
        iters = 0
        for _ in range(e_steps):
            r = mc.hcluster(Xn, Ch, msr=2, eps=0.0, maxiter=E2E_ITERS - 1, precision=args.precision, ctx=ctx)
            iters += int(r["numiter"])
        t = time.perf_counter() - t0
        e2e = {"value": iters / t, "unit": "iters/s", "h2d_bytes_per_step": int(n * D * 4 + K * D * 4),
               "d2h_bytes_per_step": int(K * D * 4 + n * 4 + n * 8),
               "call": "minicore_gb300.hcluster(host pinned rows, maxiter=9, eps=0)"}

    cpu = None
    if not args.no_cpu and rank == 0:
        threads = os.cpu_count() or 1
        S = 20_000
        Xs = X[:S].cpu().numpy()
        Cs = C0.cpu().numpy()
        per = cpu_baseline(Xs, Cs, threads)
        cpu = {"value": 1.0 / (per * n / S), "unit": "iters/s", "cores": threads, "kind": "port",
               "sample": f"{S} rows x k={K}: one assignment + centroid update of the oracle, scaled by {n}/{S}"}

    serving = None
    if not args.no_serving and rank == 0:
        del job
        torch.cuda.synchronize()
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
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk,
                "job_latency_ms": (serving or {}).get("latency_ms"),
                "serving": serving}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
