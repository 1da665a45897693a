"""The serving path on the GPU: jobs seeded on the device (mc_job_create_kmeanspp) and the
continuous-batching server (mc_server_*).

Bars: a job seeded on the device gives the same center ids, assignments, centers and costs
as kmeanspp followed by hcluster (and as the oracle for dense SQRL2); every job served in a
mix of concurrent jobs gives bit-for-bit the results it gives when it runs alone.
"""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mc():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import minicore_gb300
    return minicore_gb300


def _mixture(n, d, k, seed, nonneg=False):
    rng = np.random.default_rng(seed)
    mu = rng.uniform(-10, 10, (k, d))
    X = mu[rng.integers(0, k, n)] + rng.normal(size=(n, d))
    if nonneg:
        X = np.abs(X)
    return X.astype(np.float32)


def _counts(n, d, density, seed):
    rng = np.random.default_rng(seed)
    M = sp.random(n, d, density=density, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.integers(1, 6, s).astype(np.float32)).tolil()
    for i in range(n):
        if M.rows[i] == []:
            M[i, int(rng.integers(0, d))] = 1.0
    M = M.tocsr()
    M.sort_indices()
    return M.astype(np.float32)


def _job_outputs(job, n, d):
    C = np.empty((job.k, d), np.float32)
    asn = np.empty(n, np.uint32)
    costs = np.empty(n, np.float64)
    job.read(C, asn, costs)
    return C, asn, costs


def test_job_from_kmeanspp_matches_kmeanspp_then_hcluster(mc, orc):
    X = _mixture(6000, 24, 12, seed=3)
    seed = 1234
    job = mc.Job.from_kmeanspp(X, 12, msr=2, seed=seed)
    ids, _, _ = mc.kmeanspp(X, 12, msr=2, seed=seed)
    assert np.array_equal(job.center_ids, ids)
    ic, fc, it = job.run(eps=0.0, maxiter=9)
    C, asn, costs = _job_outputs(job, *X.shape)
    res = mc.hcluster(X, ids.astype(np.int64), msr=2, eps=0.0, maxiter=9, seed=seed)
    assert (ic, fc, it) == (res["initcost"], res["finalcost"], res["numiter"])
    assert np.array_equal(asn, res["asn"]) and np.array_equal(C, res["centers"])
    # and the oracle's kmeans++ then EM on the same uniforms
    oids, _, _ = orc.kmeanspp(X, 12, 2, 0.0, orc.uniforms(seed, 12))
    assert np.array_equal(oids, ids)
    ores = orc.hcluster(X, X[oids.astype(np.int64)], 2, 0.0, eps=0.0, maxiter=9, seed=seed)
    assert np.array_equal(asn, ores["asn"]) and np.array_equal(C, ores["centers"])
    assert fc == ores["finalcost"]


def test_job_from_kmeanspp_csr_and_errors(mc):
    X = _counts(1500, 300, 0.05, seed=4)
    job = mc.Job.from_kmeanspp(X, 7, msr=5, prior=1.0, seed=99)
    ids, _, _ = mc.kmeanspp(X, 7, msr=5, prior=1.0, seed=99)
    assert np.array_equal(job.center_ids, ids)
    ic, fc, it = job.run(eps=1e-10, maxiter=5)
    res = mc.hcluster(X, ids.astype(np.int64), msr=5, prior=1.0, eps=1e-10, maxiter=5, seed=99)
    assert (ic, fc, it) == (res["initcost"], res["finalcost"], res["numiter"])
    _, asn, _ = _job_outputs(job, *X.shape)
    assert np.array_equal(asn, res["asn"])
    with pytest.raises(ValueError):
        mc.Job.from_kmeanspp(X[:5], 6, msr=5, prior=1.0, seed=1)


def _mix():
    """A mix of job kinds: dense SQRL2 FP32 / BF16 / TF32, dense L1, JSD and Hellinger,
    CSR MKL and SQRL2; explicit centers and device seeding."""
    jobs = []
    for i in range(4):
        X = _mixture(3000 + 1700 * i, 16 << (i % 3), 5 + 3 * i, seed=100 + i)
        jobs.append(dict(matrix=X, k=5 + 3 * i, msr=2, precision=["fp32", "bf16", "tf32", "bf16"][i],
                         seed=7 + i, eps=1e-10, maxiter=12))
    P = _mixture(2500, 12, 4, seed=200, nonneg=True)
    jobs.append(dict(matrix=P, centers=P[:4].copy(), msr=0, seed=3, eps=1e-10, maxiter=6))
    jobs.append(dict(matrix=P, k=4, msr=4, prior=1.0, seed=4, eps=1e-10, maxiter=6))
    jobs.append(dict(matrix=P, k=6, msr=6, prior=0.0, seed=5, eps=1e-10, maxiter=6))
    for i in range(3):
        S = _counts(1200 + 600 * i, 500, 0.02, seed=300 + i)
        jobs.append(dict(matrix=S, k=6 + i, msr=5, prior=1.0, seed=11 + i, eps=1e-10, maxiter=8))
    S = _counts(1800, 300, 0.03, seed=400)
    jobs.append(dict(matrix=S, centers=np.arange(0, 1800, 200), msr=2, seed=12, eps=1e-10, maxiter=8))
    return jobs


def _same(a, b):
    for key in ("initcost", "finalcost", "numiter"):
        assert a[key] == b[key], key
    for key in ("centers", "asn", "costs", "center_ids"):
        if key in a or key in b:
            assert np.array_equal(a[key], b[key]), key


def test_server_same_result_alone_and_in_the_mix(mc):
    jobs = _mix()
    alone = []
    with mc.Server(slots=1) as srv:
        for j in jobs:
            alone.append(srv.wait(srv.submit(**j)))
    with mc.Server(slots=4) as srv:
        tickets = [srv.submit(**j) for j in jobs]
        # twice the mix, submitted back to back, so the slots stay full
        tickets += [srv.submit(**j) for j in jobs]
        mixed = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == 2 * len(jobs) and st["failed"] == 0
    assert st["max_running"] >= 2
    for i, r in enumerate(mixed):
        _same(alone[i % len(jobs)], r)
    # the served job equals the library's one-call form
    j = jobs[0]
    ids, _, _ = mc.kmeanspp(j["matrix"], j["k"], msr=2, seed=j["seed"])
    res = mc.hcluster(j["matrix"], ids.astype(np.int64), msr=2, eps=j["eps"], maxiter=j["maxiter"],
                      seed=j["seed"], precision=j["precision"])
    assert np.array_equal(alone[0]["center_ids"], ids)
    assert np.array_equal(alone[0]["asn"], res["asn"])
    assert alone[0]["finalcost"] == res["finalcost"]


def test_server_admission_budget_serializes(mc):
    jobs = _mix()[:5]
    # a budget smaller than any job: only a job that would run alone is admitted
    with mc.Server(slots=4, mem_budget=1) as srv:
        ts = [srv.submit(**j) for j in jobs]
        out = [srv.wait(t) for t in ts]
        st = srv.stats()
    assert st["max_running"] == 1 and st["completed"] == len(jobs)
    assert all(r["queue_ms"] >= 0 and r["run_ms"] > 0 and r["total_ms"] >= r["run_ms"] for r in out)


def test_server_failures_and_poll(mc):
    X = _mixture(800, 8, 3, seed=9)
    # column index out of range in row 2: rejected by the CSR check on the device
    bad = mc.CSparseMatrix(data=np.ones(6, np.float32), indices=np.array([0, 1, 999, 3, 4, 5], np.uint32),
                           indptr=np.arange(7, dtype=np.uint64), shape=(6, 6))
    with mc.Server(slots=2) as srv:
        with pytest.raises(NotImplementedError):
            srv.submit(X, k=3, msr=1)
        with pytest.raises(ValueError):
            srv.submit(X[:2], k=3)
        tb = srv.submit(bad, centers=np.eye(6, dtype=np.float32)[:2], msr=2)
        tg = srv.submit(X, k=3, seed=5, maxiter=4)
        with pytest.raises(Exception) as ei:
            srv.wait(tb)
        assert "index" in str(ei.value).lower() or "csr" in str(ei.value).lower()
        r = None
        for _ in range(100000):
            r = srv.poll(tg)
            if r is not None:
                break
        if r is None:
            r = srv.wait(tg)
        assert r["numiter"] >= 1 and r["asn"].shape == (800,)
        st = srv.stats()
        assert st["failed"] == 1 and st["completed"] == 1
        assert st["p50_total_ms"] > 0 and st["p99_total_ms"] >= st["p50_total_ms"]
        with pytest.raises(ValueError):
            srv.wait(tg)  # the ticket was released with its result
