"""The three ways of running the Lloyd loop give the same results: the host loop (a round
trip per decision), the fused loop (device-side stop rule, a round trip per iteration) and
the CUDA graph (while-conditional node, a round trip per run): same iterations, objective,
centers, assignments and costs, on the tensor-core, FP32 tiled and CSR sparse-dot paths,
with weights, with an empty-cluster restart (the device loops hand back to the host and
resume) and with eps = 0 (the loop runs until the objective rises and the last update is
reverted)."""
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
    yield minicore_gb300
    minicore_gb300.loop_mode(minicore_gb300.LOOP_AUTO)


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


def _both(mc, X, centers, **kw):
    """Host loop result, and the fused and graph results checked equal to it."""
    mc.loop_mode(mc.LOOP_HOST)
    a = mc.hcluster(X, centers, **kw)
    out = []
    for mode in (mc.LOOP_FUSED, mc.LOOP_GRAPH):
        mc.loop_mode(mode)
        l0 = mc.kernel_launches()
        out.append(mc.hcluster(X, centers, **kw))
        assert mc.kernel_launches() > l0
    mc.loop_mode(mc.LOOP_AUTO)
    _same(a, out[0])
    return a, out[1]


def _same(a, b):
    assert a["numiter"] == b["numiter"]
    assert a["initcost"] == b["initcost"] and a["finalcost"] == b["finalcost"]
    assert np.array_equal(a["asn"], b["asn"])
    assert np.array_equal(a["costs"], b["costs"], equal_nan=True)
    ca, cb = a["centers"], b["centers"]
    if isinstance(ca, tuple):
        for u, v in zip(ca[0], cb[0]):
            assert np.array_equal(u, v)
    else:
        assert np.array_equal(ca, cb)


@pytest.mark.parametrize("precision", ["bf16", "tf32", "fp32"])
def test_dense_sqrl2_graph_equals_host_loop(mc, precision):
    X = _mixture(20000, 64, 30, seed=1)
    ids, _, _ = mc.kmeanspp(X, 30, msr=2, seed=5)
    a, b = _both(mc, X, ids.astype(np.int64), msr=2, eps=1e-6, maxiter=25, precision=precision)
    _same(a, b)
    assert a["numiter"] >= 2


def test_eps_zero_runs_to_revert(mc):
    X = _mixture(6000, 16, 12, seed=2)
    a, b = _both(mc, X, X[:12].copy(), msr=2, eps=0.0, maxiter=300, precision="bf16")
    _same(a, b)


@pytest.mark.parametrize("msr", [0, 4, 5, 6])
def test_dense_other_measures_weighted(mc, msr):
    X = _mixture(5000, 24, 8, seed=10 + msr, nonneg=True)
    w = np.random.default_rng(msr).random(5000) + 0.5
    a, b = _both(mc, X, X[:8].copy(), msr=msr, prior=1.0, weights=w, eps=1e-8, maxiter=15)
    _same(a, b)


@pytest.mark.parametrize("msr", [5, 4, 2])
def test_csr_graph_equals_host_loop(mc, msr):
    X = _counts(4000, 100, 0.2, seed=msr)
    ids = np.arange(0, 4000, 400)
    a, b = _both(mc, X, ids, msr=msr, prior=1.0, eps=1e-8, maxiter=12)
    _same(a, b)


def test_empty_cluster_restart_then_graph_resumes(mc):
    X = _mixture(8000, 8, 6, seed=31)
    C0 = np.concatenate([X[:6], np.full((2, 8), 1e3, np.float32)])
    a, b = _both(mc, X, C0, msr=2, eps=0.0, maxiter=8, seed=77)
    _same(a, b)
    assert a["numiter"] >= 3
