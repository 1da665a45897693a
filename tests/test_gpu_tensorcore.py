"""tcgen05 BF16 / TF32 SQRL2 assignment against the exact FP32 path and the oracle.

The rounding bound plus the exact FP32 re-check of candidate rows make the tensor-core
assignment identical to the FP32 assignment on every row (assignment indices bit-exact,
costs bit-exact: the cost is always the exact sequential FP32 distance).
"""
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


def _assign(mc, X, C, precision):
    from minicore_gb300 import _lib
    M = mc._MatrixArg(X)
    C = np.ascontiguousarray(C, np.float32)
    asn = np.empty(M.n, np.uint32)
    costs = np.empty(M.n, np.float64)
    _lib.check(_lib.load().mc_assign(mc.default_context().handle, M.ref, mc._p(C), C.shape[0], 2, 0.0,
                                     mc._PREC[precision], mc._p(asn), mc._p(costs)))
    return asn, costs


def _data(n, d, k, seed, dup_frac=0.3):
    rng = np.random.default_rng(seed)
    comps = max(2, k // 2)
    mu = rng.normal(size=(comps, d)) * 2.0
    X = (mu[rng.integers(0, comps, n)] + rng.normal(size=(n, d))).astype(np.float32)
    C = X[rng.choice(n, k, replace=False)].copy()
    # near-duplicate centers create rows with margins below the bound
    nd = int(dup_frac * k)
    if nd:
        C[:nd] = C[k - nd:] + rng.normal(size=(nd, d)).astype(np.float32) * 0.05
    return X, C


@pytest.mark.parametrize("precision", ["bf16", "tf32"])
def test_tc_small_matches_fp32(mc, orc, precision):
    X, C = _data(1000, 128, 300, seed=1)
    a32, c32 = _assign(mc, X, C, "fp32")
    atc, ctc = _assign(mc, X, C, precision)
    assert np.array_equal(atc, a32)
    assert np.array_equal(ctc, c32)
    oa, oc = orc.assign(X, C, 2, 0.0)
    assert np.array_equal(atc, oa)
    assert np.array_equal(ctc, oc)


@pytest.mark.parametrize("precision", ["bf16", "tf32"])
@pytest.mark.parametrize("n,d,k", [(20000, 128, 1024), (7777, 50, 37), (5000, 200, 257), (3000, 64, 1),
                                   (4099, 33, 513)])
def test_tc_matches_fp32(mc, precision, n, d, k):
    X, C = _data(n, d, k, seed=n + d + k)
    a32, c32 = _assign(mc, X, C, "fp32")
    atc, ctc = _assign(mc, X, C, precision)
    assert np.array_equal(atc, a32)
    assert np.array_equal(ctc, c32)


def test_tc_recheck_fraction_and_hcluster(mc, orc):
    rng = np.random.default_rng(4)
    mu = rng.normal(size=(64, 128)) * 2.0
    X = (mu[rng.integers(0, 64, 30000)] + rng.normal(size=(30000, 128))).astype(np.float32)
    ids, _, _ = mc.kmeanspp(X, 64, msr=2, seed=9)
    r32 = mc.hcluster(X, ids.astype(np.int64), msr=2, eps=0.0, maxiter=5, seed=1, precision="fp32")
    for prec in ("bf16", "tf32"):
        r = mc.hcluster(X, ids.astype(np.int64), msr=2, eps=0.0, maxiter=5, seed=1, precision=prec)
        assert r["numiter"] == r32["numiter"]
        assert np.array_equal(r["asn"], r32["asn"])
        assert np.array_equal(r["centers"], r32["centers"])
        assert r["finalcost"] == r32["finalcost"]
    j = mc.Job(X, X[ids.astype(np.int64)], msr=2, precision="bf16")
    j.assign()
    assert j.recheck_count() < 0.5 * len(X)


def test_tc_nan_rows(mc):
    X, C = _data(2000, 64, 40, seed=3)
    X[5, 3] = np.nan
    a32, c32 = _assign(mc, X, C, "fp32")
    atc, ctc = _assign(mc, X, C, "bf16")
    assert np.array_equal(atc, a32)
    assert np.array_equal(ctc[np.isfinite(c32)], c32[np.isfinite(c32)])
    assert np.isnan(ctc[5]) == np.isnan(c32[5])


def test_tc_bounded_wait_expires_and_context_survives(mc):
    """The device failure path, without faulting anything: the test hook makes pass 1's MMA
    issuer wait on a barrier that nothing completes.  Its bound (about one second) runs out,
    the kernel drains its copies in flight, frees its tensor memory and returns; the call
    reports MC_ETIMEOUT, and the next call on the same context gives the FP32 result."""
    import time
    from minicore_gb300 import _lib
    lib = _lib.load()
    X, C = _data(4096, 64, 256, seed=11)
    a32, c32 = _assign(mc, X, C, "fp32")
    M = mc._MatrixArg(X)
    asn = np.empty(M.n, np.uint32)
    costs = np.empty(M.n, np.float64)
    assert lib.mc_test_tc_stall_once() == _lib.MC_OK
    t0 = time.perf_counter()
    rc = lib.mc_assign(mc.default_context().handle, M.ref, mc._p(C), C.shape[0], 2, 0.0, _lib.MC_BF16,
                       mc._p(asn), mc._p(costs))
    waited = time.perf_counter() - t0
    assert rc == _lib.MC_ETIMEOUT, lib.mc_last_error()
    assert b"bounded wait expired" in lib.mc_last_error()
    assert waited < 30.0
    for _ in range(2):  # the hook is one shot; the context is intact
        atc, ctc = _assign(mc, X, C, "bf16")
        assert np.array_equal(atc, a32)
        assert np.array_equal(ctc, c32)
