"""Soft clustering (perform_soft_clustering, solve.h:287-374) on the GPU against the oracle.

Bars: relative 1e-5 on objectives and centers, 1e-5 absolute on soft assignments, equal
iteration counts (CUDA expf and glibc expf may differ in the last ulp)."""
import numpy as np
import pytest

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
    mu = rng.uniform(-4, 4, (k, d))
    X = mu[rng.integers(0, k, n)] + rng.normal(size=(n, d))
    return (np.abs(X) if nonneg else X).astype(np.float32)


@pytest.mark.parametrize("msr,prior,temp", [(2, 0.0, 0.05), (2, 0.0, 1.0), (5, 1.0, 2.0), (6, 1.0, 3.0)])
@pytest.mark.parametrize("weighted", [False, True])
def test_scluster_matches_oracle(mc, orc, msr, prior, temp, weighted):
    X = _mixture(2500, 10, 6, seed=msr * 10 + int(temp * 10), nonneg=msr != 2)
    C0 = X[:6].copy()
    w = np.random.default_rng(8).uniform(0.5, 2.0, len(X)) if weighted else None
    g = mc.scluster(X, C0, msr=msr, prior=prior, temp=temp, maxiter=6, weights=w)
    o = orc.scluster(X, C0, msr, prior, weights=w, temp=temp, maxiter=6)
    assert g["numiter"] == o["numiter"]
    np.testing.assert_allclose(g["initcost"], o["initcost"], rtol=1e-5)
    np.testing.assert_allclose(g["finalcost"], o["finalcost"], rtol=1e-5)
    np.testing.assert_allclose(g["centers"], o["centers"], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(g["asn"], o["asn"], atol=1e-5)
    np.testing.assert_allclose(g["costs"], o["costs"], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(g["asn"].sum(1), 1.0, rtol=1e-5)


def test_cluster_soft_entry(mc):
    X = _mixture(1500, 8, 4, seed=1)
    r = mc.cluster(X, msr=2, k=4, temp=0.5, maxiter=5, seed=3)
    assert r["asn"].shape == (1500, 4) and r["centers"].shape == (4, 8)


@pytest.mark.parametrize("msr,prior,temp", [(2, 0.0, 0.5), (5, 1.0, 2.0), (6, 1.0, 1.0)])
@pytest.mark.parametrize("weighted", [False, True])
def test_scluster_csr_matches_oracle(mc, orc, msr, prior, temp, weighted):
    """CSR rows: the soft means accumulate over each row's nonzeros (a zero adds nothing to
    the compensated sums); distances come from the CSR assignment kernels."""
    import scipy.sparse as sp
    rng = np.random.default_rng(30 + msr)
    X = sp.random(1800, 120, density=0.08, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.integers(1, 6, s).astype(np.float32)).astype(np.float32)
    X.sort_indices()
    C0 = np.asarray(X[rng.choice(1800, 5, replace=False)].toarray(), np.float32) + 0.1
    w = rng.uniform(0.5, 2.0, 1800) if weighted else None
    g = mc.scluster(X, C0, msr=msr, prior=prior, temp=temp, maxiter=5, weights=w)
    o = orc.scluster(X, C0, msr, prior, weights=w, temp=temp, maxiter=5)
    assert g["numiter"] == o["numiter"]
    np.testing.assert_allclose(g["initcost"], o["initcost"], rtol=1e-4)
    np.testing.assert_allclose(g["finalcost"], o["finalcost"], rtol=1e-4)
    (data, idx, indptr), shape = g["centers"]
    Cg = sp.csr_matrix((data, idx.astype(np.int64), indptr.astype(np.int64)), shape=tuple(shape)).toarray()
    np.testing.assert_allclose(Cg, o["centers"], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(g["asn"], o["asn"], atol=1e-4)


@pytest.mark.parametrize("temp", [0.3, 4.0])
@pytest.mark.parametrize("weighted", [False, True])
def test_scluster_l1_matches_oracle(mc, orc, temp, weighted):
    """L1 soft centers: weighted_median with the soft assignments (times the row weights) as
    weights keeps, per column, the smallest value among the rows of largest weight
    (centroid.h:815-838, kmedian.h:266-297).  Centers are copied values, so they match
    exactly whenever the soft assignments pick the same rows."""
    X = _mixture(2000, 12, 5, seed=40 + int(temp), nonneg=False)
    C0 = X[:5].copy()
    w = np.random.default_rng(9).uniform(0.5, 2.0, len(X)) if weighted else None
    g = mc.scluster(X, C0, msr=0, temp=temp, maxiter=5, weights=w)
    o = orc.scluster(X, C0, 0, 0.0, weights=w, temp=temp, maxiter=5)
    assert g["numiter"] == o["numiter"]
    np.testing.assert_allclose(g["finalcost"], o["finalcost"], rtol=1e-5)
    np.testing.assert_array_equal(g["centers"], o["centers"])
    np.testing.assert_allclose(g["asn"], o["asn"], atol=1e-5)
    # every center coordinate is a value of the matrix's column
    for c in g["centers"]:
        assert all(np.any(X[:, j] == c[j]) for j in range(X.shape[1]))


def test_scluster_l1_csr_raises(mc):
    import scipy.sparse as sp
    X = sp.random(200, 30, density=0.2, format="csr", random_state=1, dtype=np.float32)
    with pytest.raises(Exception, match="weighted L1 median"):
        mc.scluster(X, X[:3].toarray(), msr=0, temp=1.0, maxiter=2)
