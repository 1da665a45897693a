"""CPU checks of the FP64 references that bench.py's accuracy blocks use: the MKL and JSD
identities of fp64_csr_distances against a direct float64 evaluation over every column,
and the SQRL2 check against float64 differences."""
import os
import sys

import numpy as np
import scipy.sparse as sp

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _direct(msr, X, C):
    """KL(c~ || p~) and JSD(c~, p~) over all columns in float64 (prior 1)."""
    X = np.asarray(X, np.float64)
    C = np.asarray(C, np.float64)
    d = X.shape[1]
    p = (X + 1.0) / (X.sum(1, keepdims=True) + d)
    c = (C + 1.0) / (C.sum(1, keepdims=True) + d)
    out = np.empty((X.shape[0], C.shape[0]))
    for i in range(X.shape[0]):
        a, b = c, p[i][None, :]
        if msr == 5:
            out[i] = (a * np.log(a / b)).sum(1)
        else:
            m = 0.5 * (a + b)
            out[i] = 0.5 * ((a * np.log(a / m)).sum(1) + (b * np.log(b / m)).sum(1))
    return np.maximum(out, 0.0)


def test_fp64_csr_identities_match_direct_evaluation():
    rng = np.random.default_rng(0)
    X = sp.random(60, 300, density=0.05, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.integers(1, 9, s).astype(np.float32))
    X.sort_indices()
    C = rng.random((7, 300)).astype(np.float32) * (rng.random((7, 300)) < 0.3)
    for msr in (5, 4):
        got = bench.fp64_csr_distances(msr, X, C)
        want = _direct(msr, X.toarray(), C)
        np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-13)


def test_fp64_sqrl2_check():
    rng = np.random.default_rng(1)
    X = rng.normal(size=(500, 16)).astype(np.float32)
    C = rng.normal(size=(9, 16)).astype(np.float32)
    D = ((X[:, None, :].astype(np.float64) - C[None].astype(np.float64)) ** 2).sum(2)
    asn = D.argmin(1).astype(np.uint32)
    r = bench.fp64_sqrl2_check(X, C, asn, D.min(1))
    assert r["argmin_agreement"] == 1.0 and r["rel_err"] < 1e-12
