"""Pairwise distance matrices (cmp / pcmp) on the GPU against the oracle's per-pair distances.

Bars: dense SQRL2, L1 and Hellinger bit-exact (the same sequential FP32 expression as the
oracle); dense MKL/JSD relative 2e-5 (logf may differ by an ulp); CSR rows relative 1e-4
(the GPU evaluates CSR rows by the algebraic decompositions of the sparse sums).
"""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

EXACT = {0, 2, 6}


@pytest.fixture(scope="module")
def mc():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import minicore_gb300
    return minicore_gb300


def _data(n, d, seed, nonneg=True):
    rng = np.random.default_rng(seed)
    X = rng.gamma(2.0, 1.0, (n, d)) if nonneg else rng.normal(size=(n, d))
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


def _check(got, want, msr, sparse):
    if msr in EXACT and not sparse:
        assert np.array_equal(got, want)
    else:
        np.testing.assert_allclose(got, want, rtol=1e-4 if sparse else 2e-5, atol=1e-6)


@pytest.mark.parametrize("msr", [0, 2, 4, 5, 6])
@pytest.mark.parametrize("prior", [0.0, 1.0])
def test_cmp_dense_both_roles(mc, orc, msr, prior):
    X, Y = _data(70, 24, 1 + msr), _data(9, 24, 50 + msr)
    got = mc.cmp(X, Y, msr=msr, prior=prior)
    want = np.array([[orc.msr_dense(msr, X[i], Y[j], prior) for j in range(9)] for i in range(70)], np.float32)
    _check(got, want, msr, False)
    got_r = mc.cmp(X, Y, msr=msr, prior=prior, reverse=False)
    want_r = np.array([[orc.msr_dense(msr, Y[j], X[i], prior) for j in range(9)] for i in range(70)], np.float32)
    _check(got_r, want_r, msr, False)
    v = mc.cmp(X, Y[3], msr=msr, prior=prior)
    assert v.shape == (70,)
    _check(v, want[:, 3], msr, False)
    assert isinstance(mc.cmp(X[0], Y[0], msr=msr, prior=prior), float)


@pytest.mark.parametrize("msr", [0, 2, 4, 5, 6])
def test_cmp_csr(mc, orc, msr):
    X = _counts(60, 300, 0.05, seed=msr)
    Y = np.asarray(_counts(7, 300, 0.08, seed=90 + msr).toarray(), np.float32) + 0.25
    got = mc.cmp(X, Y, msr=msr, prior=1.0)
    Xd = X.toarray()
    want = np.array([[orc.msr_sparse(msr, Xd[i], Y[j], 1.0) for j in range(7)] for i in range(60)], np.float32)
    _check(got, want, msr, True)


@pytest.mark.parametrize("msr", [0, 2, 5, 6])
def test_pcmp_dense_and_csr(mc, orc, msr):
    X = _data(40, 16, 7 + msr)
    got = mc.pcmp(X, msr=msr, prior=1.0)
    n = len(X)
    want = np.array([orc.msr_dense(msr, X[j], X[i], 1.0) for i in range(n) for j in range(i + 1, n)], np.float32)
    assert got.shape == (n * (n - 1) // 2,)
    _check(got, want, msr, False)
    S = _counts(30, 200, 0.06, seed=msr)
    gs = mc.pcmp(S, msr=msr, prior=1.0)
    Sd = S.toarray()
    ws = np.array([orc.msr_sparse(msr, Sd[j], Sd[i], 1.0) for i in range(30) for j in range(i + 1, 30)], np.float32)
    np.testing.assert_allclose(gs, ws, rtol=1e-4, atol=1e-6)


def test_cmp_errors(mc):
    X = _data(10, 5, 0)
    with pytest.raises(ValueError):
        mc.cmp(X, _data(3, 6, 1))
    with pytest.raises(NotImplementedError):
        mc.cmp(X, _data(3, 5, 1), msr=1)
    assert mc.pcmp(X[:1]).shape == (0,)
