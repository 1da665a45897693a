"""The oracle against the reference's own known-answer tests and invariants.

Anchors: src/tests/testmsr.cpp (self-distance ~0 for every measure and prior in
{0, 1, 50, 1e-2}; positivity of msr(cv1, cv4); the MKL value for prior 1),
src/tests/testmsrcsr.cpp (sparse and dense representations agree within 1e-5 on the large
count-vector pair), src/tests/test_centroid.cpp (exact weighted means), and
src/tests/coreset_test.cpp (sampled indices in range).
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

GOLD = os.path.join(os.path.dirname(__file__), "golden", "msr_fixtures.npz")
MEASURES = [0, 2, 4, 5, 6]  # L1, SQRL2, JSD, MKL, HELLINGER


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("msr", MEASURES)
@pytest.mark.parametrize("prior", [0.0, 1.0, 50.0, 1e-2])
def test_self_distance_zero_and_positive(orc, gold, msr, prior):
    cv1, cv4 = gold["cv1"], gold["cv4"]
    for f in (orc.msr_dense, orc.msr_sparse):
        v = f(msr, cv1, cv1, prior)
        assert abs(v) <= 5e-4  # testmsr.cpp:50-55
        assert not np.isnan(v)
        assert f(msr, cv1, cv4, prior) > 0  # testmsr.cpp:62-66


def test_mkl_known_answer(orc, gold):
    # testmsr.cpp:67 calls msr_with_prior(MKL, cv1, cv4, prior=1, psum=12, ...).
    # The reference's own sparse correction terms (applicator.h:1849) fix the direction as
    # KL(center~ || row~) with the 3rd argument (cv4) as the center: 0.5377195590904397.
    # The value printed by that test, 0.539179777847523, is the other direction.
    cv1, cv4 = gold["cv1"], gold["cv4"]
    v = orc.msr_dense(5, cv1, cv4, 1.0, 12.0)
    assert v == pytest.approx(0.5377195590904397, rel=2e-6)
    assert orc.msr_sparse(5, cv1, cv4, 1.0, 12.0) == pytest.approx(0.5377195590904397, rel=2e-6)
    a = (cv4.astype(np.float64) + 1) / (cv4.sum() + 12)
    b = (cv1.astype(np.float64) + 1) / (cv1.sum() + 12)
    assert float((b * np.log(b / a)).sum()) == pytest.approx(0.539179777847523, rel=1e-12)


def test_large_sparse_pair_dense_vs_sparse(orc, gold):
    d = int(gold["big_dim"])
    lhs = np.zeros(d, np.float32)
    rhs = np.zeros(d, np.float32)
    lhs[gold["lhs_idx"]] = gold["lhs_val"]
    rhs[gold["rhs_idx"]] = gold["rhs_val"]
    prior = 1e-5  # testmsr.cpp:72-73
    for msr in (5,):
        v_dense = orc.msr_dense(msr, lhs, rhs, prior, prior * d)
        v_sparse = orc.msr_sparse(msr, lhs, rhs, prior, prior * d)
        assert v_dense > 0 and v_sparse > 0
        assert abs(v_dense - v_sparse) <= 1e-5 * max(1.0, abs(v_dense))  # testmsrcsr.cpp:94-95
    for msr in MEASURES:
        a = orc.msr_dense(msr, lhs, rhs, 1.0)
        b = orc.msr_sparse(msr, lhs, rhs, 1.0)
        assert abs(a - b) <= 1e-5 * max(1.0, abs(a))


def _np_measure(msr, row, cen, prior):
    """FP64 textbook form of each measure (applicator.h:1672-1760)."""
    row = row.astype(np.float64)
    cen = cen.astype(np.float64)
    d = row.size
    pv = prior
    a = (cen + pv) / (cen.sum() + pv * d)
    b = (row + pv) / (row.sum() + pv * d)
    if msr == 2:
        return ((cen - row) ** 2).sum()
    if msr == 0:
        return np.abs(cen - row).sum()
    if msr == 6:
        return np.sqrt(((np.sqrt(a) - np.sqrt(b)) ** 2).sum()) * np.sqrt(0.5)
    if msr == 5:
        return (a * np.log(a / b)).sum()
    if msr == 4:
        m = a + b
        return 0.5 * (a * np.log(a) + b * np.log(b) - m * np.log(m / 2)).sum()


@pytest.mark.parametrize("msr", MEASURES)
def test_measures_match_fp64_formulas(orc, msr):
    rng = np.random.default_rng(5)
    for _ in range(20):
        d = int(rng.integers(3, 300))
        row = rng.poisson(2.0, d).astype(np.float32)
        cen = rng.gamma(2.0, 1.0, d).astype(np.float32)
        for prior in (0.5, 1.0):
            ref = _np_measure(msr, row, cen, prior)
            assert orc.msr_dense(msr, row, cen, prior) == pytest.approx(ref, rel=2e-5, abs=1e-6)
            assert orc.msr_sparse(msr, row, cen, prior) == pytest.approx(ref, rel=2e-5, abs=1e-6)


def test_centroid_known_answers(orc):
    # test_centroid.cpp:48-60: identity-diagonal rows (value 10 on the diagonal) -> mean 1;
    # 10x10 CSR diagonal of ones -> 0.1 everywhere.
    dm = np.eye(10, dtype=np.float32) * 10
    out = orc.hcluster(dm, dm[:1], 2, 0.0, maxiter=0)  # one center: the mean of all rows
    # after one update the single center is the column mean
    Xs = sp.csr_matrix(np.eye(10, dtype=np.float32))
    res = orc.hcluster(Xs, np.eye(10, dtype=np.float32)[:1], 2, 0.0, maxiter=0)
    assert np.allclose(res["centers"][0], 0.1, atol=1e-7)
    # fcsm2 case (test_centroid.cpp:94-112): rows i have columns 0,2,4,6,8 with values
    # 2(5i+j+1); the mean of column 2j is 47 + 2j.
    data = 2.0 * (np.arange(50) + 1.0)
    idx = np.tile(np.arange(0, 10, 2), 10)
    indptr = np.arange(0, 51, 5)
    F = sp.csr_matrix((data.astype(np.float32), idx, indptr), shape=(10, 10))
    res = orc.hcluster(F, F.toarray()[:1], 2, 0.0, maxiter=0)
    c = res["centers"][0]
    for j in range(5):
        assert int(c[2 * j]) == 47 + 2 * j


def test_det_sum_and_draw(orc):
    rng = np.random.default_rng(1)
    v = rng.random(100_003)
    assert orc.det_sum(v) == pytest.approx(v.sum(), rel=1e-13)
    # canonical order: the elements in index order (pairwise trees inside 8192-element
    # chunks and over the chunk totals)
    n = v.size
    order = np.arange(n)
    pos = np.arange(n)
    c = np.cumsum(v[order])
    for u in rng.random(200):
        i = orc.det_draw(v, u)
        t = u * c[-1]
        # the drawn element's cumulative interval contains the target (up to rounding)
        p = pos[i]
        lo = c[p - 1] if p else 0.0
        assert lo - 1e-9 * c[-1] <= t <= c[p] + 1e-9 * c[-1]
    z = np.zeros(10)
    assert orc.det_draw(z, 0.5) == 10
    w = np.zeros(20000)
    w[12345] = 3.0
    assert orc.det_draw(w, 0.999) == 12345
    assert orc.det_draw(w, 0.0) == 12345


def test_det_sum_is_the_pairwise_tree(orc):
    """The canonical sum: pairwise over consecutive elements inside 8192-element chunks,
    then pairwise over the chunk totals padded with zeros to a power of two."""
    rng = np.random.default_rng(5)
    for n in (1, 31, 8192, 8193, 3 * 8192 + 17, 100_003):
        v = rng.random(n) * 10.0 ** rng.integers(-8, 8, n)

        def pairwise(x):
            x = list(x)
            while len(x) > 1:
                x = [x[i] + x[i + 1] for i in range(0, len(x), 2)]
            return x[0]

        G = -(-n // 8192)
        pad = np.zeros(G * 8192)
        pad[:n] = v
        tot = [pairwise(pad[g * 8192:(g + 1) * 8192]) for g in range(G)]
        P = 1
        while P < G:
            P *= 2
        assert orc.det_sum(v) == pairwise(tot + [0.0] * (P - G))


def test_uniform_stream_properties(orc):
    u = orc.uniforms(42, 100000)
    assert u.min() >= 0 and u.max() < 1
    assert abs(u.mean() - 0.5) < 0.01
    assert np.array_equal(orc.uniforms(42, 10, offset=5), u[5:15])


def test_kmeanspp_basic(orc):
    rng = np.random.default_rng(0)
    centers = rng.uniform(-10, 10, (5, 8))
    X = (centers[rng.integers(0, 5, 2000)] + rng.normal(size=(2000, 8))).astype(np.float32)
    u = orc.uniforms(7, 5)
    ids, asn, costs = orc.kmeanspp(X, 5, 2, 0.0, u)
    assert len(set(ids.tolist())) == 5
    assert costs[ids].max() == 0
    d2 = ((X[:, None, :].astype(np.float64) - X[ids][None].astype(np.float64)) ** 2).sum(-1)
    assert np.allclose(costs, d2.min(1), rtol=1e-5, atol=1e-4)
    # D^2 seeding on well-separated blobs hits every blob in most runs
    true = ((X[:, None] - centers[None]) ** 2).sum(-1).argmin(1)
    hits = sum(len(set(true[orc.kmeanspp(X, 5, 2, 0.0, orc.uniforms(s, 5))[0]].tolist())) == 5
               for s in range(20))
    assert hits >= 15


def test_hcluster_converges_monotone(orc):
    rng = np.random.default_rng(3)
    mu = rng.uniform(-10, 10, (25, 50))
    X = (mu[np.repeat(np.arange(25), 40)] + rng.normal(size=(1000, 50))).astype(np.float32)
    u = orc.uniforms(11, 25)
    ids, _, _ = orc.kmeanspp(X, 25, 2, 0.0, u)
    res = orc.hcluster(X, X[ids], 2, 0.0, maxiter=19)
    assert res["finalcost"] <= res["initcost"]
    d2 = ((X[:, None, :].astype(np.float64) - res["centers"][None].astype(np.float64)) ** 2).sum(-1)
    assert np.array_equal(res["asn"], d2.argmin(1))


@pytest.mark.parametrize("method", [0, 1, 2, 3, 4])
def test_sensitivity_and_sampling(orc, method):
    rng = np.random.default_rng(method)
    n, nc = 10000, 20
    asn = rng.integers(0, nc, n).astype(np.uint32)
    costs = (rng.integers(0, 3, n) + 0.1).astype(np.float32)
    w = (1.0 / (rng.integers(0, 5, n) + 1)).astype(np.float32)
    for weights in (None, w):
        p = orc.sensitivity(costs, asn, nc, method, weights=weights)
        assert np.all(p > 0)
        if method != 1:
            assert p.astype(np.float64).sum() == pytest.approx(1.0, rel=1e-5)
        pt, at = orc.alias_build(p)
        for m in (20, 200, 2000):
            wo, io = orc.coreset_sample(p, pt, at, m, seed=9, weights=weights, method=method, b=nc)
            assert io.max() < n  # coreset_test.cpp:30
            wo2, io2 = orc.coreset_sample(p, pt, at, m, seed=9, unique=True, weights=weights, method=method, b=nc)
            direct = m - nc if method == 1 else m
            assert np.all(np.diff(io2[:direct].astype(np.int64)) > 0)


def test_alias_table_is_exact_distribution(orc):
    rng = np.random.default_rng(2)
    p = rng.random(1000).astype(np.float32) ** 3
    pt, at = orc.alias_build(p)
    n = p.size
    mass = pt / n
    mass_alias = np.zeros(n)
    np.add.at(mass_alias, at, (1 - pt) / n)
    q = p.astype(np.float64) / p.astype(np.float64).sum()
    assert np.allclose(mass + mass_alias, q, atol=1e-12)


def test_oracle_l1_centers_are_medians(orc):
    """set_centroids_l1 restated: after an update every L1 center is the coordinate-wise
    median of its rows (even sizes: 0.5f * (the two middles)); with weights, the value of the
    largest-weight row (the reference's weighted_median never accumulates its total)."""
    rng = np.random.default_rng(12)
    X = (rng.normal(size=(400, 5)) * 3).astype(np.float32)
    C0 = X[[0, 100, 200, 300]].copy()
    r = orc.hcluster(X, C0, 0, 0.0, eps=0.0, maxiter=0, seed=1)
    # maxiter 0: one update; rows reassigned to the medians of the first assignment
    a0, _ = orc.assign(X, C0, 0, 0.0)
    for c in range(4):
        col = np.sort(X[a0 == c], axis=0)
        m = col.shape[0]
        med = col[m // 2] if m % 2 else np.float32(0.5) * (col[m // 2 - 1] + col[m // 2])
        assert np.array_equal(r["centers"][c], med.astype(np.float32))
    w = rng.integers(1, 4, 400).astype(np.float64)
    cw = orc.l1_centers(X, a0, 4, weights=w)
    cu = orc.l1_centers(X, a0, 4)
    for c in range(4):
        sel = a0 == c
        top = sel & (w == w[sel].max())
        assert np.array_equal(cw[c], X[top].min(axis=0))
        assert np.array_equal(cu[c], r["centers"][c])


@pytest.mark.parametrize("weighted", [False, True])
def test_oracle_soft_l1_centers_rule(orc, weighted):
    """One soft L1 iteration: each center coordinate is the smallest column value among the
    rows whose soft weight (asn column times the row weight) is largest, the result of
    kmedian.h:266-297 (weighted_median with wsum never accumulated)."""
    rng = np.random.default_rng(5)
    X = rng.normal(size=(300, 6)).astype(np.float32)
    C0 = X[:3].copy()
    w = rng.uniform(0.5, 2.0, 300) if weighted else None
    r = orc.scluster(X, C0, 0, 0.0, weights=w, temp=0.7, maxiter=1)
    asn = r["asn"].astype(np.float64)
    for c in range(3):
        cw = asn[:, c] * (w if weighted else 1.0)
        rows = cw == cw.max()
        np.testing.assert_array_equal(r["centers"][c], X[rows].min(axis=0))
    with pytest.raises(ValueError):
        orc.scluster(sp.random(50, 6, density=0.3, format="csr", random_state=1, dtype=np.float32),
                     C0, 0, 0.0, temp=1.0, maxiter=1)


# (rows in the cluster, nonzeros of column 0, expected center value) read off the sparse
# median of util/csc.h:856-890: h = rows // 2; with more than h nonzeros of one sign the
# positive case counts the zeros first (t = h - (rows - nel)) and the negative case reads
# position rows - h; an even count averages positions t and t + 1; mixed signs sort the zeros
# in; an odd count with exactly h nonzeros of one sign gives half the extreme one.
SPARSE_MEDIAN_CASES = [
    (5, [3, 1, 2], 1.0),          # zeros, zeros, 1, 2, 3 -> 1
    (4, [1, 2, 3, 4], 3.5),       # positions 2 and 3
    (4, [5, 7, 9], 8.0),          # t = 1 -> (7 + 9) / 2
    (5, [4, 6], 2.0),             # nel == h, odd: half the smallest
    (5, [-4, -6], -2.0),          # nel == h, odd: half the largest
    (5, [-1, 2], 0.0),            # nel == h, mixed signs
    (3, [-3, -1, -2], -1.0),      # all negative, odd: position rows - h = 2
    (4, [-1, 3, 2], 2.5),         # mixed: -1 0 2 3 -> positions 2, 3
    (5, [1], 0.0),                # too few nonzeros
    (2, [1, 3], 3.0),             # position 2 runs past the end: the last element
    (6, [2, 2, 2, 2, 9], 2.0),    # t = 3 - 1 = 2 -> (2 + 2) / 2
    (7, [-5, -4, -3, -2, -1], -1.0),  # all negative, odd: position 7 - 3 = 4 (not -2)
]


@pytest.mark.parametrize("nrows,vals,expected", SPARSE_MEDIAN_CASES)
def test_oracle_sparse_l1_median_rule(orc, nrows, vals, expected):
    X = np.zeros((nrows, 3), np.float32)
    X[:len(vals), 0] = vals
    X[:, 2] = 1.0  # a column with every row equal
    S = sp.csr_matrix(X)
    c = orc.l1_centers(S, np.zeros(nrows, np.uint32), 1)
    assert c[0, 0] == np.float32(expected)
    assert c[0, 1] == 0.0 and c[0, 2] == 1.0


def test_oracle_sparse_l1_weighted_raises(orc):
    S = sp.csr_matrix(np.eye(4, dtype=np.float32))
    with pytest.raises(ValueError):
        orc.l1_centers(S, np.zeros(4, np.uint32), 1, weights=np.ones(4))


def _sparse_median_py(vals, nrows):
    """util/csc.h:856-890 for one column of one cluster, in plain Python: vals = the
    cluster's nonzeros in that column, nrows = the cluster's rows (positions past the end of
    a vector, undefined in the reference, take its last element)."""
    v = sorted(np.float32(x) for x in vals)
    nel, h = len(v), nrows // 2
    at = lambda a, q: a[min(q, len(a) - 1)]
    half = lambda a, b: np.float32(np.float32(a + b) * np.float32(0.5))
    if nel > h:
        if v[0] > 0 or v[-1] < 0:
            t = h - (nrows - nel) if v[0] > 0 else nrows - h
            return at(v, t) if nrows & 1 else half(at(v, t), at(v, t + 1))
        f = sorted(v + [np.float32(0)] * (nrows - nel))
        return f[h] if nrows & 1 else half(at(f, h), at(f, h + 1))
    if nrows & 1 and nel == h:
        if v[0] > 0:
            return np.float32(np.float32(0.5) * v[0])
        if v[-1] < 0:
            return np.float32(np.float32(0.5) * v[-1])
    return np.float32(0)


@pytest.mark.parametrize("seed", range(6))
def test_oracle_sparse_l1_medians_match_python_restatement(orc, seed):
    rng = np.random.default_rng(seed)
    n, d, k = int(rng.integers(5, 60)), int(rng.integers(1, 12)), int(rng.integers(1, 6))
    dens = rng.uniform(0.1, 0.9)
    X = (rng.integers(-3, 5, (n, d)) * (rng.random((n, d)) < dens)).astype(np.float32)
    asn = rng.integers(0, k, n).astype(np.uint32)
    asn[:k] = np.arange(k)  # no empty cluster
    S = sp.csr_matrix(X)
    got = orc.l1_centers(S, asn, k)
    for c in range(k):
        rows = np.nonzero(asn == c)[0]
        for j in range(d):
            if rows.size == 1:
                want = X[rows[0], j]
            else:
                col = S[rows][:, j].toarray().ravel()
                nz = [x for x, r in zip(col, rows) if S[r, j] != 0 or (S[r].indices == j).any()]
                want = _sparse_median_py(nz, rows.size)
            assert got[c, j] == want, (c, j)
