"""Minibatch hard clustering (perform_hard_minibatch_clustering, solve.h:386-582) on the GPU
against the oracle's restatement with the same sample streams.

Bars: dense SQRL2 bit-exact (centers, assignments, costs, objectives, iterations) in FP32 and
BF16 (the tensor-core check-ins return the FP32 assignment); CSR MKL within 1e-4 relative."""
import math

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


def _mixture(n, d, k, seed):
    rng = np.random.default_rng(seed)
    mu = rng.uniform(-10, 10, (k, d))
    return (mu[rng.integers(0, k, n)] + rng.normal(size=(n, d))).astype(np.float32)


def _same(g, o):
    assert g["numiter"] == o["numiter"]
    assert g["initcost"] == o["initcost"] and g["finalcost"] == o["finalcost"]
    assert np.array_equal(g["centers"], o["centers"])
    assert np.array_equal(g["asn"], o["asn"])
    assert np.array_equal(g["costs"].astype(np.float32), o["costs"].astype(np.float32))


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
@pytest.mark.parametrize("with_rep", [False, True])
def test_minibatch_dense_sqrl2_bit_exact(mc, orc, precision, with_rep):
    X = _mixture(6000, 20, 10, seed=3)
    C0 = X[:10].copy()
    maxiter, nchk = 25, 5
    g = mc.hcluster(X, C0, msr=2, mbsize=400, maxiter=maxiter, ncheckins=nchk, reseed_count=1,
                    with_rep=with_rep, seed=17, precision=precision)
    o = orc.minibatch(X, C0, 2, 0.0, mbsize=400, maxiter=maxiter, freq=math.ceil(maxiter / nchk), reseed_after=1,
                      with_rep=with_rep, seed=17)
    _same(g, o)
    assert g["finalcost"] <= g["initcost"]


def test_minibatch_weighted_and_restarts(mc, orc):
    X = _mixture(3000, 12, 6, seed=5)
    w = np.random.default_rng(1).uniform(0.5, 2.0, 3000)
    # two far centers and a high reseed threshold force restarts at the check-ins
    C0 = np.concatenate([X[:6], np.full((2, 12), 500.0, np.float32)])
    g = mc.hcluster(X, C0, msr=2, weights=w, mbsize=256, maxiter=12, ncheckins=4, reseed_count=40, seed=9)
    o = orc.minibatch(X, C0, 2, 0.0, weights=w, mbsize=256, maxiter=12, freq=3, reseed_after=40, seed=9)
    _same(g, o)


def test_minibatch_csr_mkl(mc, orc):
    rng = np.random.default_rng(2)
    M = sp.random(2500, 300, density=0.05, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.integers(1, 6, s).astype(np.float32)).tolil()
    for i in range(2500):
        if M.rows[i] == []:
            M[i, int(rng.integers(0, 300))] = 1.0
    M = M.tocsr().astype(np.float32)
    M.sort_indices()
    ids = np.arange(0, 2500, 500)
    C0 = np.asarray(M[ids].toarray(), np.float32)
    g = mc.hcluster(M, ids, msr=5, prior=1.0, mbsize=300, maxiter=10, ncheckins=2, reseed_count=1, seed=4)
    o = orc.minibatch(M, C0, 5, 1.0, mbsize=300, maxiter=10, freq=5, reseed_after=1, seed=4)
    assert g["numiter"] == o["numiter"]
    np.testing.assert_allclose(g["finalcost"], o["finalcost"], rtol=1e-4)
    np.testing.assert_allclose(g["initcost"], o["initcost"], rtol=1e-4)
    assert (g["asn"] == o["asn"]).mean() > 0.99


@pytest.mark.parametrize("msr,weighted,precision", [(2, False, "fp32"), (2, True, "fp32"), (2, False, "bf16"),
                                                    (0, False, "fp32")])
def test_coreset_minibatch_matches_oracle(mc, orc, msr, weighted, precision):
    """cs=True: minibatch-by-coreset EM (hmb_coreset_clustering) against the oracle's
    restatement: best centers, last assignment and costs, objectives and rounds bit for bit
    (SQRL2 in FP32 and BF16, which give the FP32 assignment; L1 with VX sensitivities and
    median centers)."""
    rng = np.random.default_rng(40 + msr)
    mu = rng.uniform(-8, 8, (6, 8))
    X = (mu[rng.integers(0, 6, 3000)] + rng.normal(size=(3000, 8))).astype(np.float32)
    C0 = X[rng.choice(3000, 6, replace=False)].copy()
    w = rng.integers(1, 4, 3000).astype(np.float64) if weighted else None
    res = mc.hcluster(X, C0, msr=msr, weights=w, mbsize=500, maxiter=20, ncheckins=5, reseed_count=1, seed=13,
                      cs=True, precision=precision)
    best, asn, costs, ic, fc, it = orc.coreset_minibatch(X, C0, msr, 0.0, 500, 20, ncheckins=5, reseed_count=1,
                                                         seed=13, weights=w)
    assert res["numiter"] == it
    assert res["initcost"] == ic and res["finalcost"] == fc
    assert np.array_equal(res["asn"], asn)
    assert np.array_equal(res["costs"], costs.astype(np.float32))
    assert np.array_equal(res["centers"], best)


@pytest.mark.parametrize("weighted", [False, True])
def test_minibatch_dense_l1_medians(mc, orc, weighted):
    """L1 minibatch: each hit center becomes the l1_median of its sampled rows (solve.h:559-561);
    with weights, weighted_median over rows(data, asp, nasn) reads the full weight vector at
    the group position (kmedian.h:329-344)."""
    X = _mixture(3000, 10, 6, seed=8)
    C0 = X[:6].copy()
    w = np.random.default_rng(4).integers(1, 5, 3000).astype(np.float64) if weighted else None
    g = mc.hcluster(X, C0, msr=0, weights=w, mbsize=301, maxiter=12, ncheckins=3, reseed_count=1, seed=6)
    o = orc.minibatch(X, C0, 0, 0.0, weights=w, mbsize=301, maxiter=12, freq=4, reseed_after=1, seed=6)
    _same(g, o)


def test_minibatch_csr_l1_medians(mc, orc):
    rng = np.random.default_rng(12)
    M = sp.random(2000, 90, density=0.1, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.integers(1, 6, s).astype(np.float32)).astype(np.float32)
    M.sort_indices()
    ids = np.arange(0, 2000, 250)
    C0 = np.asarray(M[ids].toarray(), np.float32)
    g = mc.hcluster(M, ids, msr=0, mbsize=400, maxiter=10, ncheckins=2, reseed_count=1, seed=3)
    o = orc.minibatch(M, C0, 0, 0.0, mbsize=400, maxiter=10, freq=5, reseed_after=1, seed=3)
    assert g["numiter"] == o["numiter"]
    assert g["finalcost"] == o["finalcost"]
    assert np.array_equal(g["asn"], o["asn"])
    (data, idx, indptr), shape = g["centers"]
    Cg = sp.csr_matrix((data, idx.astype(np.int64), indptr.astype(np.int64)), shape=tuple(shape)).toarray()
    assert np.array_equal(Cg, o["centers"])
