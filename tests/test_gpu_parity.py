"""GPU parity: the CUDA path (through the C ABI) against the oracle on the same seeded inputs.

Bars: integer/index results (assignments, center ids, sampled indices) bit-exact; FP32
distances bit-exact where both sides evaluate the same sequential float expression (dense
SQRL2, L1, Hellinger), otherwise within the tolerance stated per test; FP64 sums exact where
the canonical order is shared.
"""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

MEASURES = [0, 2, 4, 5, 6]
LOG_MEASURES = {4, 5}  # logf on the GPU and in glibc may differ in the last ulp
REL = 2e-5             # distance tolerance for measures with logarithms / decompositions


@pytest.fixture(scope="module")
def mc():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import minicore_gb300
    return minicore_gb300


def _mixture(n, d, k, seed, spread=10.0, nonneg=False):
    rng = np.random.default_rng(seed)
    mu = rng.uniform(-spread, spread, (k, d))
    X = mu[rng.integers(0, k, n)] + rng.normal(size=(n, d))
    if nonneg:
        X = np.abs(X)
    return X.astype(np.float32)


def _counts(n, d, density, seed):
    rng = np.random.default_rng(seed)
    M = sp.random(n, d, density=density, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.integers(1, 6, s).astype(np.float32))
    M.sort_indices()
    # every row non-empty
    M = M.tolil()
    for i in range(n):
        if M.rows[i] == []:
            M[i, int(rng.integers(0, d))] = 1.0
    M = M.tocsr()
    M.sort_indices()
    return M.astype(np.float32)


def _assign_gpu(mc, X, C, msr, prior, precision="fp32"):
    import ctypes
    from minicore_gb300 import _lib
    M = mc._MatrixArg(X)
    C = np.ascontiguousarray(C, np.float32)
    asn = np.empty(M.n, np.uint32)
    costs = np.empty(M.n, np.float64)
    _lib.check(_lib.load().mc_assign(mc.default_context().handle, M.ref, mc._p(C), C.shape[0], msr, prior,
                                     mc._PREC[precision], mc._p(asn), mc._p(costs)))
    return asn, costs


def _check_assign(orc, X, C, msr, prior, asn, costs, exact):
    oasn, ocost = orc.assign(X, C, msr, prior)
    if exact:
        assert np.array_equal(asn, oasn)
        assert np.array_equal(costs, ocost)
        return
    np.testing.assert_allclose(costs, ocost, rtol=REL, atol=1e-6)
    diff = asn != oasn
    if diff.any():
        # only near-ties may differ: the oracle's distance to our center equals its best
        Xd = X.toarray() if sp.issparse(X) else X
        for i in np.nonzero(diff)[0][:50]:
            d_ours = orc.msr_dense(msr, Xd[i], C[asn[i]], prior) if not sp.issparse(X) else \
                orc.msr_sparse(msr, Xd[i], C[asn[i]], prior)
            assert d_ours <= ocost[i] * (1 + 10 * REL) + 1e-6
        assert diff.mean() < 1e-3


def _replay_draws(mc, orc, S, k, msr, prior, seed, weights=None):
    """The D^2 draws, bit for bit, given the GPU's own distances: round c of a k-center
    run draws from the distances left by the first c centers, which the c-center run returns
    as its costs (the same uniforms U(seed, i) drive every run).  So the c-center run's ids
    must be the k-center run's first c ids, and the oracle's draw (the pairwise-tree inverse
    CDF over w * distance, with kmeans.h:179-186's argmax fallback) over those costs with
    U(seed, c) must give the k-center run's id c.  The distances themselves are checked
    against the oracle separately (they may differ in the last ulps: the GPU evaluates the
    CSR measures through algebraic decompositions)."""
    ids, _, _ = mc.kmeanspp(S, k, msr=msr, prior=prior, seed=seed, weights=weights)
    u = orc.uniforms(seed, k)
    n = S.shape[0]
    assert ids[0] == min(int(u[0] * n), n - 1)
    for c in range(1, k):
        ids_c, _, costs_c = mc.kmeanspp(S, c, msr=msr, prior=prior, seed=seed, weights=weights)
        assert np.array_equal(ids_c, ids[:c]), (c, ids_c, ids[:c])
        costs_c = np.asarray(costs_c, np.float64)
        v = costs_c if weights is None else np.asarray(weights, np.float64) * costs_c
        want = orc.det_draw(v, float(u[c]))
        if want >= n or costs_c[want] == 0.0:
            want = int(np.argmax(costs_c))
        assert want == ids[c], (c, want, ids[c])
    return ids


def _check_seed_costs(orc, S, ids, costs, msr, prior):
    """kmeans++ costs: the oracle's distance from every row to its nearest chosen row."""
    C = np.asarray(S[ids.astype(np.int64)].toarray(), np.float32)
    _, oc = orc.assign(S, C, msr, prior)
    np.testing.assert_allclose(costs, oc, rtol=1e-4, atol=1e-5)


def _check_loop_asn(orc, X, msr, prior, asn, ocenters, oasn, tol=1e-4):
    """Rows a Lloyd run assigns differently from the oracle's run must be near-ties: under
    the oracle's final centers, the row's distance to the center the GPU picked is within
    `tol` (relative) of its distance to the oracle's pick."""
    diff = np.nonzero(asn != oasn)[0]
    Xd = X.toarray() if sp.issparse(X) else X
    f = orc.msr_sparse if sp.issparse(X) else orc.msr_dense
    for i in diff:
        d_g = f(msr, Xd[i], ocenters[asn[i]], prior)
        d_o = f(msr, Xd[i], ocenters[oasn[i]], prior)
        assert d_g <= d_o * (1 + tol) + 1e-6, (i, d_g, d_o)
    assert diff.size <= max(2, X.shape[0] // 1000)


@pytest.mark.parametrize("msr", MEASURES)
@pytest.mark.parametrize("prior", [0.0, 1.0])
def test_dense_assign_matches_oracle(mc, orc, msr, prior):
    X = _mixture(3000, 37, 9, seed=msr, nonneg=msr != 2)
    rng = np.random.default_rng(100 + msr)
    C = X[rng.choice(len(X), 13, replace=False)] + 0.01
    asn, costs = _assign_gpu(mc, X, C, msr, prior)
    _check_assign(orc, X, C, msr, prior, asn, costs, exact=msr not in LOG_MEASURES)


@pytest.mark.parametrize("msr", MEASURES)
@pytest.mark.parametrize("prior", [0.0, 1.0])
def test_csr_assign_matches_oracle(mc, orc, msr, prior):
    X = _counts(1500, 300, 0.05, seed=msr)
    rng = np.random.default_rng(7 + msr)
    ids = rng.choice(X.shape[0], 7, replace=False)
    C = np.asarray(X[ids].toarray(), np.float32)
    C[:, ::7] += 0.5  # dense-ish centers, as means are
    asn, costs = _assign_gpu(mc, X, C, msr, prior)
    _check_assign(orc, X, C, msr, prior, asn, costs, exact=False)


@pytest.mark.parametrize("k", [7, 50, 130])
def test_csr_jsd_grouped_sparse_dot(mc, orc, k):
    """CSR JSD with a constant prior on count rows: rows with equal row sums share one
    zero-entry sum per center, the rest is a sparse dot (k = 50 also runs the two-rows-per-
    warp kernel); checked against the oracle's union walk, and the sparse-dot kernels ran."""
    X = _counts(4000, 100, 0.2, seed=k)   # ~100 distinct row sums, table <= nnz / 2
    rng = np.random.default_rng(k)
    C = np.asarray(X[rng.choice(4000, k, replace=False)].toarray(), np.float32)
    C[:, ::5] += 0.5
    mc.autotune(True)
    mc.autotune_reset()
    asn, costs = _assign_gpu(mc, X, C, 4, 1.0)
    _check_assign(orc, X, C, 4, 1.0, asn, costs, exact=False)
    assert any(key.startswith("csr_sparse|msr4|") for key in mc.autotune_report()["entries"])
    mc.autotune_reset()


def test_csr_jsd_real_valued_rows_fall_back(mc, orc):
    """Real-valued rows have (almost) no equal row sums: the grouping is dropped and the
    tiled column loop runs; results still match the oracle."""
    rng = np.random.default_rng(3)
    X = sp.random(1500, 200, density=0.05, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.random(s).astype(np.float32) * 4).astype(np.float32)
    X.sort_indices()
    C = np.asarray(X[rng.choice(1500, 6, replace=False)].toarray(), np.float32) + 0.1
    mc.autotune(True)
    mc.autotune_reset()
    asn, costs = _assign_gpu(mc, X, C, 4, 1.0)
    _check_assign(orc, X, C, 4, 1.0, asn, costs, exact=False)
    assert not any(key.startswith("csr_sparse|msr4|") for key in mc.autotune_report()["entries"])


def test_assign_edge_cases(mc, orc):
    # k = 1, ragged d, a single row, duplicate centers (ties -> lowest index)
    X = _mixture(257, 5, 3, seed=1)
    C = X[:1].copy()
    asn, costs = _assign_gpu(mc, X, C, 2, 0.0)
    assert np.all(asn == 0)
    _check_assign(orc, X, C, 2, 0.0, asn, costs, exact=True)
    C2 = np.concatenate([X[3:4], X[3:4], X[7:8]])
    asn, costs = _assign_gpu(mc, X, C2, 2, 0.0)
    assert not np.any(asn == 1)  # exact ties resolve to the lower index
    _check_assign(orc, X, C2, 2, 0.0, asn, costs, exact=True)
    asn, costs = _assign_gpu(mc, X[:1], C2, 2, 0.0)
    _check_assign(orc, X[:1], C2, 2, 0.0, asn, costs, exact=True)
    # many centers (several center tiles)
    C3 = X[np.random.default_rng(0).choice(257, 200, replace=False)]
    asn, costs = _assign_gpu(mc, X, C3, 2, 0.0)
    _check_assign(orc, X, C3, 2, 0.0, asn, costs, exact=True)


@pytest.mark.parametrize("msr", MEASURES)
def test_kmeanspp_dense_matches_oracle(mc, orc, msr):
    X = _mixture(4000, 24, 12, seed=3 + msr, nonneg=msr != 2)
    prior = 0.5
    k = 12
    seed = 1234 + msr
    ids, asn, costs = mc.kmeanspp(X, k, msr=msr, prior=prior, seed=seed)
    oids, oasn, ocosts = orc.kmeanspp(X, k, msr, prior, orc.uniforms(seed, k))
    assert np.array_equal(ids, oids)
    assert np.array_equal(asn.astype(np.uint32), oasn)
    if msr in LOG_MEASURES:
        np.testing.assert_allclose(costs, ocosts.astype(np.float32), rtol=REL, atol=1e-6)
    else:
        assert np.array_equal(costs, ocosts.astype(np.float32))


@pytest.mark.parametrize("weighted", [False, True])
@pytest.mark.parametrize("d", [32, 61, 64])
def test_kmeanspp_dense_sqrl2_pruned_matches_oracle(mc, orc, weighted, d, tmp_path):
    """Over large dense SQRL2 matrices (beyond the persistent-cluster sizes) the rounds may
    skip rows whose distance to the new center provably cannot beat their current one, an
    autotuner choice ("kmpp_prune"): variant 1 by the triangle inequality with FP32 rounding
    bounds, variant 2 (d = 8 G, G a power of two up to 32) by a lower bound from a BF16 copy
    of the rows (the rows it cannot settle get the exact update), variant 0 neither; each is
    forced here through a loaded decision, and ids, assignments and costs stay bit-identical
    to the oracle, which evaluates every row.  Well-separated components (most rows settled
    in later rounds), duplicated rows (zero distances), d not a multiple of 4 (the unstaged
    kernel, no BF16 screen)."""
    n = 300_000 if d == 32 else 140_000
    X = _mixture(n, d, 60, seed=d, spread=20.0)
    X[1000:1200] = X[0]
    w = np.random.default_rng(d).random(n) + 0.05 if weighted else None
    oids, oasn, ocosts = orc.kmeanspp(X, 48, 2, 0.0, orc.uniforms(77, 48), weights=w)
    mc.autotune(True)
    mc.autotune_reset()
    mc.kmeanspp(X, 48, msr=2, seed=77, weights=w)   # records the decision
    keys = [k for k in mc.autotune_report()["entries"] if k.startswith("kmpp_prune|")]
    assert len(keys) == 1
    nvar = len(mc.autotune_report()["entries"][keys[0]]["ms"])
    assert nvar == (3 if d in (32, 64) else 2)
    for v in range(nvar):
        mc.autotune_reset()
        path = tmp_path / f"prune{v}.tsv"
        path.write_text(f"{keys[0]}\t{v}\t\n")
        mc.autotune_load(str(path))
        ids, asn, costs = mc.kmeanspp(X, 48, msr=2, seed=77, weights=w)
        assert mc.autotune_report()["entries"][keys[0]]["variant"] == v
        assert np.array_equal(ids, oids)
        assert np.array_equal(asn.astype(np.uint32), oasn)
        assert np.array_equal(costs, ocosts.astype(np.float32))
    mc.autotune_reset()


@pytest.mark.parametrize("msr,trials,weighted", [(2, 3, False), (2, 2, True), (0, 4, False)])
def test_kmeanspp_greedy_matches_oracle(mc, orc, msr, trials, weighted):
    """n_local_trials > 1 (greedy seeding, kmeans.h:79-177): ids, assignments and distances
    bit-exact against the oracle's restatement."""
    X = _mixture(3000, 12, 9, seed=50 + msr, nonneg=msr != 2)
    w = np.random.default_rng(6).uniform(0.5, 2.0, 3000) if weighted else None
    ids, asn, costs = mc.kmeanspp(X, 10, msr=msr, seed=21, n_local_trials=trials, weights=w)
    oids, oasn, ocosts = orc.kmeanspp_greedy(X, 10, msr, 0.0, trials, 21, weights=w)
    assert np.array_equal(ids, oids)
    assert np.array_equal(asn.astype(np.uint32), oasn)
    assert np.array_equal(costs, ocosts.astype(np.float32))


@pytest.mark.parametrize("msr,trials,weighted", [(2, 1, False), (2, 2, True), (0, 1, False), (6, 1, False)])
def test_kmeanspp_lspp_matches_oracle(mc, orc, msr, trials, weighted):
    """lspp > 0: localsearch++ rounds after the seeding, against the oracle's restatement
    run on the same seeds (ids, assignments, costs bit for bit)."""
    X = _mixture(2500, 10, 8, seed=60 + msr, nonneg=msr != 2)
    w = np.random.default_rng(7).uniform(0.5, 2.0, 2500) if weighted else None
    prior = 1.0 if msr == 6 else 0.0
    ids, asn, costs = mc.kmeanspp(X, 8, msr=msr, prior=prior, seed=33, n_local_trials=trials, lspp=6, weights=w)
    if trials > 1:
        sids, _, _ = orc.kmeanspp_greedy(X, 8, msr, prior, trials, 33, weights=w)
    else:
        sids, _, _ = orc.kmeanspp(X, 8, msr, prior, orc.uniforms(33, 8), weights=w)
    oids, oasn, ocosts = orc.lspp(X, sids, msr, prior, 6, 33, weights=w)
    assert np.array_equal(ids, oids)
    assert np.array_equal(asn.astype(np.uint32), oasn)
    assert np.array_equal(costs, ocosts.astype(np.float32))


def test_kmeanspp_weighted_and_csr(mc, orc):
    X = _mixture(3000, 16, 8, seed=11)
    w = np.random.default_rng(2).random(3000) + 0.1
    ids, asn, costs = mc.kmeanspp(X, 8, msr=2, seed=99, weights=w)
    oids, oasn, ocosts = orc.kmeanspp(X, 8, 2, 0.0, orc.uniforms(99, 8), weights=w)
    assert np.array_equal(ids, oids)
    assert np.array_equal(costs, ocosts.astype(np.float32))
    S = _counts(2000, 200, 0.05, seed=4)
    ws = np.random.default_rng(3).random(2000) + 0.1
    for msr in (2, 5, 4):
        for wt in (None, ws):
            ids = _replay_draws(mc, orc, S, 10, msr, 1.0, 5, weights=wt)
            ids2, asn, costs = mc.kmeanspp(S, 10, msr=msr, prior=1.0, seed=5, weights=wt)
            assert np.array_equal(ids, ids2)
            assert costs.dtype == np.float64
            _check_seed_costs(orc, S, ids, costs, msr, 1.0)


@pytest.mark.parametrize("msr,prior", [(0, 1.0), (2, 0.0), (5, 1.0), (6, 0.5), (4, 1.0), (5, 1e-44), (6, 1e-44),
                                       (4, 1e-44)])
def test_kmeanspp_csr_nnz_path(mc, orc, msr, prior):
    """CSR seeding of wide rows in O(nnz) per row (per-center FP64 constants) against the
    oracle's merge of the two sparse rows; the tiny priors move the pair to the smallest-pv
    floor, where rows take the column loop."""
    # wide rows (d > 2048 takes the O(nnz) update), 12 nonzeros each, few distinct row sums
    # (JSD groups rows by their zero-entry value)
    rng = np.random.default_rng(40 + msr)
    n, d = 2500, 2600
    cols = np.stack([np.sort(rng.choice(d, 12, replace=False)) for _ in range(n)])
    vals = np.ones((n, 12), np.float32)
    vals[:, 0] = rng.integers(1, 3, n)
    S = sp.csr_matrix((vals.ravel(), cols.ravel(), np.arange(0, 12 * n + 1, 12)), shape=(n, d)).tolil()
    for i in range(0, n, 101):
        S.rows[i], S.data[i] = [], []          # empty rows
    S = S.tocsr().astype(np.float32)
    S.sort_indices()
    if msr in (4, 5, 6) and prior < 1e-30:
        S = S[np.diff(S.indptr) > 0]           # rows with no mass have no divergence then
    ids = _replay_draws(mc, orc, S, 9, msr, prior, 17)
    _, asn, costs = mc.kmeanspp(S, 9, msr=msr, prior=prior, seed=17)
    _check_seed_costs(orc, S, ids, costs, msr, prior)
    oids, oasn, ocosts = orc.kmeanspp(S, 9, msr, prior, orc.uniforms(17, 9))
    assert ids[0] == oids[0]


@pytest.mark.parametrize("msr,prior", [(5, 1.0), (2, 0.0), (6, 1.0), (0, 1.0), (4, 1.0)])
def test_kmeanspp_csr_large_sparse_nnz_path(mc, orc, msr, prior):
    """A large sparse matrix with narrow rows (n d >= 2^25, d <= 2048, fewer than one
    nonzero in eight columns) takes the O(nnz) update: draws bit-exact given the GPU's own
    distances, distances within the CSR tolerance of the oracle's merge."""
    S = _counts(20000, 1700, 0.003, seed=60 + msr)
    ids = _replay_draws(mc, orc, S, 8, msr, prior, 21)
    _, asn, costs = mc.kmeanspp(S, 8, msr=msr, prior=prior, seed=21)
    _check_seed_costs(orc, S, ids, costs, msr, prior)


@pytest.mark.parametrize("msr,prior", [(2, 0.0), (0, 1.0)])
def test_kmeanspp_csr_fused_equals_three_launch_path(mc, msr, prior):
    """d <= 4096 runs the one-launch CSR update (center densified per CTA); one more, empty
    column (d = 4097) runs take / scatter / prep / update / zero.  For SQRL2 and L1 an empty
    column adds exactly nothing, so both give the same seeds, assignments and costs."""
    S = _counts(3000, 4096, 0.004, seed=5)
    S2 = sp.csr_matrix((S.data, S.indices, S.indptr), shape=(3000, 4097))
    a = mc.kmeanspp(S, 20, msr=msr, prior=prior, seed=8)
    b = mc.kmeanspp(S2, 20, msr=msr, prior=prior, seed=8)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def test_hcluster_dense_sqrl2_bit_exact(mc, orc):
    # the small reference configuration: 25-component mixture, kmeans++, 20 updates
    rng = np.random.default_rng(0)
    mu = rng.uniform(-10, 10, (25, 50))
    X = (mu[rng.integers(0, 25, 10000)] + rng.normal(size=(10000, 50))).astype(np.float32)
    ids, _, _ = mc.kmeanspp(X, 25, msr=2, seed=42)
    C0 = X[ids.astype(np.int64)]
    res = mc.hcluster(X, ids.astype(np.int64), msr=2, eps=0.0, maxiter=19, seed=3)
    ores = orc.hcluster(X, C0, 2, 0.0, eps=0.0, maxiter=19, seed=3)
    assert res["numiter"] == ores["numiter"]
    assert np.array_equal(res["asn"], ores["asn"])
    assert np.array_equal(res["centers"], ores["centers"])
    assert np.array_equal(res["costs"], ores["costs"].astype(np.float32))
    assert res["initcost"] == ores["initcost"] and res["finalcost"] == ores["finalcost"]


@pytest.mark.parametrize("precision,msr", [("fp32", 2), ("bf16", 2), ("fp32", 5)])
def test_hcluster_f32_costs_equal_rounded_fp64_costs(mc, precision, msr):
    """mc_hcluster_f32 (the entry behind the Python hcluster) returns the same centers,
    assignments and objectives as mc_hcluster, and its costs are mc_hcluster's FP64 costs
    rounded to float32 (numpy's cast), for dense SQRL2 in both precisions and MKL."""
    import ctypes
    from minicore_gb300 import _lib
    X = _mixture(3001, 24, 7, seed=31, nonneg=msr != 2)
    C0 = X[:7].copy()
    M = mc._MatrixArg(X)
    out = {}
    for name, ctype in (("mc_hcluster", np.float64), ("mc_hcluster_f32", np.float32)):
        cout = np.empty_like(C0)
        asn = np.empty(M.n, np.uint32)
        costs = np.empty(M.n, ctype)
        ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
        _lib.check(getattr(_lib.load(), name)(mc.default_context().handle, M.ref, mc._p(C0), 7, msr, 1.0, None,
                                              0.0, 6, 5, mc._PREC[precision], mc._p(cout), mc._p(asn),
                                              mc._p(costs), ctypes.byref(ic), ctypes.byref(fc), ctypes.byref(it)))
        out[name] = (cout, asn, costs, ic.value, fc.value, it.value)
    a, b = out["mc_hcluster"], out["mc_hcluster_f32"]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[3:] == b[3:]
    assert np.array_equal(a[2].astype(np.float32), b[2])


@pytest.mark.parametrize("msr", [0, 4, 5, 6])
def test_hcluster_other_measures(mc, orc, msr):
    X = _mixture(2000, 20, 6, seed=20 + msr, nonneg=True)
    C0 = X[:6].copy()
    res = mc.hcluster(X, C0, msr=msr, prior=1.0, eps=1e-10, maxiter=8, seed=5)
    ores = orc.hcluster(X, C0, msr, 1.0, eps=1e-10, maxiter=8, seed=5)
    np.testing.assert_allclose(res["finalcost"], ores["finalcost"], rtol=1e-5)
    np.testing.assert_allclose(res["centers"], ores["centers"], rtol=1e-5, atol=1e-6)
    # hcluster returns float32 costs (pycluster.h:160): compared within the tolerance
    _check_assign(orc, X, res["centers"], msr, 1.0, res["asn"], res["costs"], exact=False)
    _check_loop_asn(orc, X, msr, 1.0, res["asn"], ores["centers"], ores["asn"])


def test_hcluster_csr_mkl(mc, orc):
    X = _counts(3000, 400, 0.04, seed=9)
    ids = np.arange(0, 3000, 300)
    C0 = np.asarray(X[ids].toarray(), np.float32)
    res = mc.hcluster(X, ids, msr=5, prior=1.0, eps=1e-10, maxiter=6, seed=1)
    ores = orc.hcluster(X, C0, 5, 1.0, eps=1e-10, maxiter=6, seed=1)
    np.testing.assert_allclose(res["finalcost"], ores["finalcost"], rtol=1e-4)
    (data, idx, indptr), shape = res["centers"]
    Cg = sp.csr_matrix((data, idx.astype(np.int64), indptr.astype(np.int64)), shape=tuple(shape)).toarray()
    np.testing.assert_allclose(Cg, ores["centers"], rtol=1e-4, atol=1e-6)
    # the final assignment is the oracle's assignment to the final centers (near-ties
    # aside), and rows the two runs assign differently are near-ties under the oracle's
    _check_assign(orc, X, Cg.astype(np.float32), 5, 1.0, res["asn"], res["costs"], exact=False)
    _check_loop_asn(orc, X, 5, 1.0, res["asn"], ores["centers"], ores["asn"])


@pytest.mark.parametrize("weighted", [False, True])
def test_hcluster_l1_medians(mc, orc, weighted):
    """L1 centers are coordinate-wise medians (set_centroids_l1): odd and even cluster sizes,
    weights (the reference's weighted_median keeps the largest-weight row's value), bit-exact
    against the oracle."""
    X = _mixture(3001, 11, 5, seed=77, nonneg=False)
    C0 = X[[0, 500, 1000, 1500, 2000, 2500]].copy()
    w = np.random.default_rng(3).integers(1, 6, 3001).astype(np.float64) if weighted else None
    res = mc.hcluster(X, C0, msr=0, prior=0.0, weights=w, eps=0.0, maxiter=6, seed=9)
    ores = orc.hcluster(X, C0, 0, 0.0, eps=0.0, maxiter=6, seed=9, weights=w)
    assert res["numiter"] == ores["numiter"]
    assert np.array_equal(res["asn"], ores["asn"])
    assert np.array_equal(res["centers"], ores["centers"])
    assert res["finalcost"] == ores["finalcost"]
    # one update from a known assignment: the GPU centers are the oracle's median rule
    a0, _ = orc.assign(X, C0, 0, 0.0)
    one = mc.hcluster(X, C0, msr=0, prior=0.0, weights=w, eps=0.0, maxiter=0, seed=9)
    if one["numiter"] == 1:
        assert np.array_equal(one["centers"], orc.l1_centers(X, a0, 6, weights=w))


def test_hcluster_l1_empty_cluster_reseed(mc, orc):
    """An L1 center far from every row: the L1 restart reseeds it by a D^2 draw and moves
    the rows that are closer in plain L1, then takes medians (oracle bit-exact)."""
    X = _mixture(2000, 6, 4, seed=5)
    C0 = np.concatenate([X[:4], np.full((1, 6), 1e4, np.float32)])
    res = mc.hcluster(X, C0, msr=0, prior=0.0, eps=0.0, maxiter=4, seed=21)
    ores = orc.hcluster(X, C0, 0, 0.0, eps=0.0, maxiter=4, seed=21)
    assert res["numiter"] == ores["numiter"]
    assert np.array_equal(res["asn"], ores["asn"])
    assert np.array_equal(res["centers"], ores["centers"])


def test_hcluster_empty_cluster_restart(mc, orc):
    # a far-away duplicate center attracts no rows -> D^2 restart path
    X = _mixture(3000, 8, 4, seed=31)
    C0 = np.concatenate([X[:4], np.full((1, 8), 1e3, np.float32)])
    res = mc.hcluster(X, C0, msr=2, eps=0.0, maxiter=4, seed=77)
    ores = orc.hcluster(X, C0, 2, 0.0, eps=0.0, maxiter=4, seed=77)
    assert res["numiter"] == ores["numiter"]
    assert np.array_equal(res["asn"], ores["asn"])
    assert np.array_equal(res["centers"], ores["centers"])


def test_hcluster_weighted(mc, orc):
    X = _mixture(5000, 12, 7, seed=41)
    w = np.random.default_rng(1).random(5000) * 3
    C0 = X[:7].copy()
    res = mc.hcluster(X, C0, msr=2, weights=w, eps=0.0, maxiter=6, seed=2)
    ores = orc.hcluster(X, C0, 2, 0.0, weights=w, eps=0.0, maxiter=6, seed=2)
    assert np.array_equal(res["asn"], ores["asn"])
    assert np.array_equal(res["centers"], ores["centers"])
    assert res["finalcost"] == ores["finalcost"]


@pytest.mark.parametrize("method", [0, 1, 2, 3, 4])
def test_coreset_sampler_bit_exact(mc, orc, method):
    rng = np.random.default_rng(method)
    n, nc = 20000, 20
    asn = rng.integers(0, nc, n).astype(np.uint32)
    costs = (rng.integers(0, 3, n) + rng.random(n)).astype(np.float32)
    w = (1.0 / (rng.integers(0, 5, n) + 1)).astype(np.float32)
    for weights in (None, w):
        cs = mc.CoresetSampler()
        cs.make_sampler(nc, costs, asn, weights=weights, sens=method)
        p = cs.get_probs()
        op = orc.sensitivity(costs, asn, nc, method, weights=weights)
        assert np.array_equal(p, op)
        pt, at = cs.alias_table()
        opt, oat = orc.alias_build(op)
        assert np.array_equal(at, oat)
        assert np.array_equal(pt, opt)
        for unique in (False, True):
            wo, io = cs.sample(3000, seed=17, unique=unique)
            owo, oio = orc.coreset_sample(op, opt, oat, 3000, seed=17, unique=unique, weights=weights,
                                          method=method, b=nc)
            assert np.array_equal(io, oio)
            assert np.array_equal(wo, owo)


def test_coreset_sampler_costs_f64_and_errors(mc, orc):
    rng = np.random.default_rng(5)
    n = 5000
    asn = rng.integers(0, 10, n).astype(np.uint32)
    costs = rng.random(n)
    cs = mc.CoresetSampler()
    cs.make_sampler(10, costs, asn, sens=4)
    assert np.array_equal(cs.get_probs(), orc.sensitivity(costs, asn, 10, 4))
    bad = asn.copy()
    bad[3] = 10
    with pytest.raises(ValueError):
        mc.CoresetSampler().make_sampler(10, costs, bad)
    with pytest.raises(ValueError):
        mc.CoresetSampler().make_sampler(10, costs.astype(np.int32), asn)


def test_det_sums_match(mc, orc):
    # objective totals share the canonical FP64 order
    X = _mixture(100_003, 4, 3, seed=8)
    C = X[:3].copy()
    j = mc.Job(X, C, msr=2)
    j.assign()
    c = j.cost()
    _, ocosts = orc.assign(X, C, 2, 0.0)
    assert c == float(np.float32(orc.det_sum(ocosts)))


def _signed_sparse(n, d, density, seed, lo=-3, hi=4):
    rng = np.random.default_rng(seed)
    M = sp.random(n, d, density=density, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.integers(lo, hi, s).astype(np.float32))
    M.sort_indices()
    return M.astype(np.float32)


def _dense_centers(res):
    (data, idx, indptr), shape = res["centers"]
    return sp.csr_matrix((data, idx.astype(np.int64), indptr.astype(np.int64)), shape=tuple(shape)).toarray()


@pytest.mark.parametrize("path", ["bucket", "sort"])
@pytest.mark.parametrize("signed", [False, True])
def test_hcluster_csr_l1_medians(mc, orc, signed, path, monkeypatch):
    """L1 over CSR rows: the sparse median rule (util/csc.h:829-893) on the device, by
    (cluster, column) buckets with a radix select, or (MC_L1CSR_SORT=1, the path for more than
    2^28 buckets) by a radix sort of all nonzeros; bit-exact against the oracle: positive
    counts, and signed values with stored zeros (every branch of the rule)."""
    if path == "sort":
        monkeypatch.setenv("MC_L1CSR_SORT", "1")
    X = _signed_sparse(1200, 60, 0.25, seed=11) if signed else _counts(1500, 80, 0.1, seed=12)
    ids = np.random.default_rng(4).choice(X.shape[0], 9, replace=False)
    C0 = np.asarray(X[ids].toarray(), np.float32)
    res = mc.hcluster(X, ids, msr=0, prior=0.0, eps=0.0, maxiter=5, seed=2)
    ores = orc.hcluster(X, C0, 0, 0.0, eps=0.0, maxiter=5, seed=2)
    assert res["numiter"] == ores["numiter"]
    assert np.array_equal(res["asn"], ores["asn"])
    assert np.array_equal(_dense_centers(res), ores["centers"])
    assert res["finalcost"] == ores["finalcost"]


def test_csr_l1_median_one_update_small_clusters(mc, orc):
    """One L1 update over CSR rows from a known assignment, with clusters of 1, 2, 3, 4 and
    more rows (the one-row copy, the m = 2 end-of-vector position, odd/even rules)."""
    X = _signed_sparse(400, 50, 0.3, seed=21, lo=-2, hi=5)
    rng = np.random.default_rng(6)
    ids = rng.choice(400, 40, replace=False)  # many centers -> small clusters
    C0 = np.asarray(X[ids].toarray(), np.float32)
    a0, _ = orc.assign(X, C0, 0, 0.0)
    sizes = np.bincount(a0, minlength=40)
    assert (sizes == 1).any() and (sizes == 2).any()
    one = mc.hcluster(X, ids, msr=0, prior=0.0, eps=0.0, maxiter=0, seed=9)
    ref = orc.l1_centers(X, a0, 40) if (sizes > 0).all() else None
    if one["numiter"] == 1 and ref is not None:
        assert np.array_equal(_dense_centers(one), ref)
    ores = orc.hcluster(X, C0, 0, 0.0, eps=0.0, maxiter=0, seed=9)
    assert one["numiter"] == ores["numiter"]
    assert np.array_equal(_dense_centers(one), ores["centers"])


def test_hcluster_csr_l1_weighted_raises(mc):
    X = _counts(300, 40, 0.2, seed=3)
    with pytest.raises(Exception, match="weighted L1 median"):
        mc.hcluster(X, np.arange(4), msr=0, weights=np.ones(300), maxiter=3)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_csr_l1_loop_modes_agree(mc, orc, mode):
    """The CSR median inside the fused loop and the CUDA-graph loop gives the host loop's
    result."""
    X = _counts(2000, 120, 0.08, seed=31)
    ids = np.arange(0, 2000, 200)
    mc.loop_mode(mode)
    try:
        res = mc.hcluster(X, ids, msr=0, prior=0.0, eps=0.0, maxiter=20, seed=5)
    finally:
        mc.loop_mode(mc.LOOP_AUTO)
    ores = orc.hcluster(X, np.asarray(X[ids].toarray(), np.float32), 0, 0.0, eps=0.0, maxiter=20, seed=5)
    assert res["numiter"] == ores["numiter"]
    assert np.array_equal(res["asn"], ores["asn"])
    assert np.array_equal(_dense_centers(res), ores["centers"])


@pytest.mark.parametrize("k", [5, 33, 70])
def test_csr_l1_prior0_union_walk_exact(mc, orc, k):
    """L1 over CSR rows with prior 0 (pair-dependent pv): the union merge walk gives the
    oracle's distances and assignments bit for bit; signed values, stored zeros, an empty row,
    values small enough for pv to matter, centers with zero columns, several lane rounds."""
    X = _signed_sparse(1500, 120, 0.12, seed=k).tolil()
    X[4, :] = 0.0
    X[9, 7] = 3e-38
    X[9, 8] = -2e-38
    X = X.tocsr()
    X.sort_indices()
    rng = np.random.default_rng(k)
    C = np.asarray(X[rng.choice(1500, k, replace=False)].toarray(), np.float32)
    C[:, ::5] += 0.25
    C[0, 7] = 1e-38
    asn, costs = _assign_gpu(mc, X, C, 0, 0.0)
    _check_assign(orc, X, C, 0, 0.0, asn, costs, exact=True)
    # the distance output of the same kernel (cmp) against the oracle's per-pair values
    D = mc.cmp(X, C, msr=0, prior=0.0)
    Xd = X.toarray()
    for i in (0, 4, 9, 777):
        for c in (0, k - 1):
            assert D[i, c] == np.float32(orc.msr_sparse(0, Xd[i], C[c], 0.0))


def test_hcluster_csr_l1_empty_cluster_reseed(mc, orc):
    """A CSR L1 center far from every row: the restart draws a row (D^2 over the costs), moves
    the rows closer to it (union walk of the two rows), then takes the sparse medians; oracle
    bit-exact."""
    X = _counts(1500, 90, 0.1, seed=44)
    C0 = np.concatenate([np.asarray(X[[3, 300, 600, 900]].toarray(), np.float32),
                         np.full((1, 90), 1e4, np.float32)])
    res = mc.hcluster(X, C0, msr=0, prior=0.0, eps=0.0, maxiter=4, seed=13)
    ores = orc.hcluster(X, C0, 0, 0.0, eps=0.0, maxiter=4, seed=13)
    assert res["numiter"] == ores["numiter"]
    assert np.array_equal(res["asn"], ores["asn"])
    assert np.array_equal(_dense_centers(res), ores["centers"])


@pytest.mark.parametrize("centers", ["dense", "disjoint"])
def test_csr_l1_prior0_walk_forms(mc, orc, centers):
    """Both walks of the CSR L1 prior-0 kernel: dense centers (every group's column union is
    every column: the warp-uniform walk) and centers with disjoint supports (the per-lane
    merge); 40 centers (two groups), empty rows, d = 97."""
    X = _signed_sparse(900, 97, 0.15, seed=61).tolil()
    X[10, :] = 0.0
    X[11, :] = 0.0
    X = X.tocsr()
    X.sort_indices()
    rng = np.random.default_rng(62)
    if centers == "dense":
        C = rng.uniform(-2, 3, (40, 97)).astype(np.float32)
    else:
        C = np.zeros((40, 97), np.float32)
        for c in range(40):
            cols = [(c * 2 + t) % 97 for t in range(2)]
            C[c, cols] = rng.uniform(0.5, 3, 2)
    asn, costs = _assign_gpu(mc, X, C, 0, 0.0)
    _check_assign(orc, X, C, 0, 0.0, asn, costs, exact=True)


def test_csr_l1_one_column_and_one_center(mc, orc):
    X = sp.csr_matrix(np.array([[1.0], [0.0], [3.0], [-2.0], [0.0]], np.float32))
    for C in (np.array([[0.5]], np.float32), np.array([[0.0], [2.0], [-1.0]], np.float32)):
        asn, costs = _assign_gpu(mc, X, C, 0, 0.0)
        _check_assign(orc, X, C, 0, 0.0, asn, costs, exact=True)
    res = mc.hcluster(X, np.array([[0.0], [2.0]], np.float32), msr=0, eps=0.0, maxiter=3, seed=1)
    ores = orc.hcluster(X, np.array([[0.0], [2.0]], np.float32), 0, 0.0, eps=0.0, maxiter=3, seed=1)
    assert res["numiter"] == ores["numiter"]
    assert np.array_equal(res["asn"], ores["asn"])
    assert np.array_equal(_dense_centers(res), ores["centers"])
