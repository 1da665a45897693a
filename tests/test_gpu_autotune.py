"""Autotuner on the GPU: every tuned family gives the same results with tuning on (variants
timed on first use) and off (defaults), and records its decision."""
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
    minicore_gb300.autotune(True)


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


def _assign(mc, X, C, msr, prior):
    import ctypes
    from minicore_gb300 import _lib
    M = mc._MatrixArg(X)
    C = np.ascontiguousarray(C, np.float32)
    asn = np.empty(M.n, np.uint32)
    costs = np.empty(M.n, np.float64)
    _lib.check(_lib.load().mc_assign(mc.default_context().handle, M.ref, mc._p(C), C.shape[0], msr, prior,
                                     mc._PREC["fp32"], mc._p(asn), mc._p(costs)))
    return asn, costs


@pytest.mark.parametrize("k", [20, 50, 150])
def test_csr_sparse_tuned_equals_default(mc, k):
    X = _counts(3000, 800, 0.03, seed=k)
    C = np.asarray(X[np.arange(0, 3000, 3000 // k)[:k]].toarray(), np.float32)
    mc.autotune(False)
    a0, c0 = _assign(mc, X, C, 5, 1.0)
    mc.autotune_reset()
    mc.autotune(True)
    a1, c1 = _assign(mc, X, C, 5, 1.0)   # tunes: every variant runs, the last one's output stays
    a2, c2 = _assign(mc, X, C, 5, 1.0)   # the kept variant
    assert np.array_equal(a0, a1) and np.array_equal(c0, c1)
    assert np.array_equal(a0, a2) and np.array_equal(c0, c2)
    ent = mc.autotune_report()["entries"]
    assert any(key.startswith("csr_sparse|msr5|") for key in ent)
    assert all(len(v["ms"]) in (3, 5, 6) and 0 <= v["variant"] < len(v["ms"])
               for key, v in ent.items() if key.startswith("csr"))


@pytest.mark.parametrize("msr,prior", [(5, 1.0), (6, 1.0), (2, 0.0), (0, 0.5), (4, 1.0)])
def test_csr_every_variant_equals_default(mc, msr, prior, tmp_path):
    """Each CSR kernel variant, forced through a loaded decision, matches variant 0 bit for bit
    (k = 50 pads to 64 centers, which adds the two-rows-per-warp kernel; odd n leaves the last
    warp a single row; empty and long rows are included)."""
    X = _counts(3001, 300, 0.12, seed=msr).tolil()
    for i in range(0, 3001, 97):
        X.rows[i], X.data[i] = [], []
    for i in range(5, 3001, 211):
        cols = np.arange(0, 300, 2)
        X.rows[i], X.data[i] = list(cols), list(np.full(cols.size, 2.0, np.float32))
    X = X.tocsr().astype(np.float32)
    X.sort_indices()
    C = np.asarray(X[np.arange(1, 3001, 60)[:50]].toarray(), np.float32) + 0.25
    mc.autotune_reset()
    mc.autotune(True)
    _assign(mc, X, C, msr, prior)
    keys = [k for k in mc.autotune_report()["entries"] if k.startswith("csr_sparse|")]
    nvar = 5 if msr == 4 else 6  # the column-band kernel covers every measure but JSD
    assert len(keys) == 1 and mc.autotune_report()["entries"][keys[0]]["ms"].__len__() == nvar
    ref = None
    for v in range(nvar):
        mc.autotune_reset()
        path = tmp_path / f"v{v}.tsv"
        path.write_text(f"{keys[0]}\t{v}\t\n")
        mc.autotune_load(str(path))
        got = _assign(mc, X, C, msr, prior)
        assert mc.autotune_report()["entries"][keys[0]]["variant"] == v
        if ref is None:
            ref = got
        assert np.array_equal(ref[0], got[0]), v
        assert np.array_equal(ref[1], got[1], equal_nan=True), v
    mc.autotune_reset()


def test_dense_sqrl2_and_kmeanspp_tuned_equal_default(mc):
    rng = np.random.default_rng(4)
    X = (rng.normal(size=(20000, 64)) + rng.integers(0, 8, (20000, 1))).astype(np.float32)
    C = X[rng.choice(20000, 256, replace=False)]
    mc.autotune(False)
    a0, c0 = _assign(mc, X, C, 2, 0.0)
    ids0, asn0, cost0 = mc.kmeanspp(X, 40, msr=2, seed=11)
    mc.autotune_reset()
    mc.autotune(True)
    for _ in range(2):
        a1, c1 = _assign(mc, X, C, 2, 0.0)
        ids1, asn1, cost1 = mc.kmeanspp(X, 40, msr=2, seed=11)
        assert np.array_equal(a0, a1) and np.array_equal(c0, c1)
        assert np.array_equal(ids0, ids1) and np.array_equal(asn0, asn1) and np.array_equal(cost0, cost1)
    keys = list(mc.autotune_report()["entries"])
    assert any(k.startswith("dense_sqrl2|dense|k256|") for k in keys)
    assert any(k.startswith("kmpp_dense|msr2|") for k in keys)


def _assign_prec(mc, X, C, precision):
    from minicore_gb300 import _lib
    M = mc._MatrixArg(X)
    C = np.ascontiguousarray(C, np.float32)
    asn = np.empty(M.n, np.uint32)
    costs = np.empty(M.n, np.float64)
    _lib.check(_lib.load().mc_assign(mc.default_context().handle, M.ref, mc._p(C), C.shape[0], 2, 0.0,
                                     mc._PREC[precision], mc._p(asn), mc._p(costs)))
    return asn, costs


@pytest.mark.parametrize("precision", ["bf16", "tf32"])
@pytest.mark.parametrize("n,d,k", [(9000, 128, 512), (5000, 96, 100), (3001, 40, 300), (6000, 128, 1280),
                                   (4000, 64, 1536), (2500, 20, 1024)])
def test_tc_every_tile_shape_equals_fp32(mc, precision, n, d, k, tmp_path):
    """Each tensor-core tile shape (BN 256 with 4 or 3 stages when the padded center count
    is a multiple of 256, BN 128 with 4 or 6 stages always), forced for both passes through a
    loaded decision, gives the FP32 path's assignments and costs bit for bit; with tuning on,
    the first call records a decision per pass.  Pass 1 has one more variant where a row is
    at most two 128-byte k-blocks and the centers fill 256-center chunks: the centers resident
    in shared memory, split into groups of 4 (one k-block) or 2 chunks, one group per CTA (the
    cases above cover one group, two and three groups, and a last group with fewer chunks)."""
    rng = np.random.default_rng(n + k)
    mu = rng.normal(size=(max(2, k // 2), d)) * 2.0
    X = (mu[rng.integers(0, mu.shape[0], n)] + rng.normal(size=(n, d))).astype(np.float32)
    C = X[rng.choice(n, k, replace=False)].copy()
    C[: k // 4] = C[k - k // 4:] + rng.normal(size=(k // 4, d)).astype(np.float32) * 0.05  # near ties
    mc.autotune(False)
    ref = _assign_prec(mc, X, C, "fp32")
    mc.autotune_reset()
    mc.autotune(True)
    got = _assign_prec(mc, X, C, precision)   # tunes both passes
    assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])
    ent = mc.autotune_report()["entries"]
    keys = {p: [kk for kk in ent if kk.startswith(f"tc{p}|{precision}|")] for p in (1, 2)}
    assert len(keys[1]) == 1 and len(keys[2]) == 1
    nvar = len(ent[keys[1][0]]["ms"])
    kp = (k + 127) // 128 * 128
    kb = -(-d * (4 if precision == "tf32" else 2) // 128)
    resident = kp % 256 == 0 and kb <= 2
    assert nvar == (4 if kp % 256 == 0 else 2) + (1 if resident else 0)
    assert len(ent[keys[2][0]]["ms"]) == (4 if kp % 256 == 0 else 2)
    for v in range(nvar):
        mc.autotune_reset()
        path = tmp_path / f"tc{v}.tsv"
        path.write_text(f"{keys[1][0]}\t{v}\t\n{keys[2][0]}\t{v}\t\n")
        mc.autotune_load(str(path))
        got = _assign_prec(mc, X, C, precision)
        assert mc.autotune_report()["entries"][keys[1][0]]["variant"] == v
        assert np.array_equal(ref[0], got[0]), v
        assert np.array_equal(ref[1], got[1]), v
    mc.autotune_reset()


@pytest.mark.parametrize("msr,prior", [(5, 1.0), (6, 1.0), (2, 0.0), (0, 0.5)])
def test_csr_band_kernel_many_bands_equals_default(mc, msr, prior, tmp_path):
    """The column-band kernel (variant 5) over 2000 columns (six 384-column bands): rows of
    100 nonzeros spread over every band, rows of 1000 (windows of 32 crossing band edges),
    empty rows, a row with one nonzero in the last column, and a row count that leaves the
    last CTA chunk partly empty; bit-identical to variant 0 and to the oracle's tolerance."""
    rng = np.random.default_rng(100 + msr)
    n, d = 2999, 2000
    X = sp.random(n, d, density=0.05, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.integers(1, 6, s).astype(np.float32)).tolil()
    for i in range(0, n, 101):
        X.rows[i], X.data[i] = [], []
    for i in range(7, n, 151):
        cols = np.sort(rng.choice(d, 1000, replace=False))
        X.rows[i], X.data[i] = list(cols), list(rng.integers(1, 6, 1000).astype(np.float32))
    X.rows[3], X.data[3] = [d - 1], [2.0]
    X = X.tocsr().astype(np.float32)
    X.sort_indices()
    C = np.asarray(X[np.arange(2, n, 60)[:50]].toarray(), np.float32) + 0.125
    mc.autotune_reset()
    mc.autotune(True)
    _assign(mc, X, C, msr, prior)
    keys = [k for k in mc.autotune_report()["entries"] if k.startswith("csr_sparse|")]
    assert len(keys) == 1
    got = {}
    for v in (0, 5):
        mc.autotune_reset()
        path = tmp_path / f"b{v}.tsv"
        path.write_text(f"{keys[0]}\t{v}\t\n")
        mc.autotune_load(str(path))
        got[v] = _assign(mc, X, C, msr, prior)
        assert mc.autotune_report()["entries"][keys[0]]["variant"] == v
    assert np.array_equal(got[0][0], got[5][0])
    assert np.array_equal(got[0][1], got[5][1], equal_nan=True)
    mc.autotune_reset()


def test_csr_l1_union_walk_variants_equal_oracle(mc, orc, tmp_path):
    """L1 over CSR rows with prior 0 (pair-dependent pv): the register-window lockstep walk
    (variant 0) and the per-row lockstep / per-lane merge kernel (variant 1), forced in turn,
    both equal the oracle's all-column walk bit for bit; rows longer than a 32-element window,
    empty rows and a union longer than 32 columns are included."""
    rng = np.random.default_rng(77)
    n, d = 1500, 700
    X = sp.random(n, d, density=0.08, format="csr", random_state=rng,
                  data_rvs=lambda s: rng.integers(1, 9, s).astype(np.float32)).tolil()
    for i in range(0, n, 89):
        X.rows[i], X.data[i] = [], []
    X = X.tocsr().astype(np.float32)
    X.sort_indices()
    C = np.asarray(X[np.arange(3, n, 40)[:37]].toarray(), np.float32)
    C[:, ::5] += 1.5
    oasn, ocost = orc.assign(X, C, 0, 0.0)
    mc.autotune_reset()
    mc.autotune(True)
    _assign(mc, X, C, 0, 0.0)
    keys = [k for k in mc.autotune_report()["entries"] if k.startswith("csr_l1_union|")]
    assert len(keys) == 1
    for v in (0, 1):
        mc.autotune_reset()
        path = tmp_path / f"l1{v}.tsv"
        path.write_text(f"{keys[0]}\t{v}\t\n")
        mc.autotune_load(str(path))
        asn, cost = _assign(mc, X, C, 0, 0.0)
        assert mc.autotune_report()["entries"][keys[0]]["variant"] == v
        assert np.array_equal(asn, oasn), v
        assert np.array_equal(cost, ocost), v
    mc.autotune_reset()


@pytest.mark.parametrize("msr,prior,weighted,n,d,k,dup", [
    (2, 0.0, False, 20011, 96, 40, False),   # three chunks, a ragged last 32-row block
    (2, 0.0, True, 9000, 64, 25, False),     # weighted draws
    (0, 0.5, False, 5003, 33, 17, False),    # L1, d not a multiple of 4 (scalar loads)
    (6, 1.0, False, 3001, 40, 10, False),    # Hellinger
    (5, 1.0, False, 4001, 52, 12, False),    # MKL
    (4, 1.0, False, 3001, 40, 10, False),    # JSD
    (2, 0.0, False, 3000, 16, 12, True),     # five distinct rows: zero total, first-maximum fallback
    (2, 0.0, False, 262144, 32, 8, False),   # 32 chunks, 2^23 values: the largest cluster case
])
def test_kmeanspp_cluster_equals_launches(mc, orc, msr, prior, weighted, n, d, k, dup, tmp_path):
    """Dense k-means++ as one persistent thread-block cluster (variant 1 of "kmpp_run") and as
    a launch sequence per round (variant 0), each forced through a loaded decision: identical
    center ids, assignments and costs, and for the exact measures identical to the oracle."""
    rng = np.random.default_rng(n + d + k)
    if msr in (4, 5, 6):
        X = rng.integers(0, 6, size=(n, d)).astype(np.float32)
    else:
        X = (rng.normal(size=(n, d)) * 3.0).astype(np.float32)
    if dup:
        X = X[rng.integers(0, 5, n)]
    w = rng.uniform(0.5, 2.0, n) if weighted else None
    mc.autotune_reset()
    mc.autotune(True)
    mc.kmeanspp(X, k, msr=msr, prior=prior, seed=5, weights=w)   # records the decision
    keys = [kk for kk in mc.autotune_report()["entries"] if kk.startswith("kmpp_run|")]
    assert len(keys) == 1
    got = []
    for v in (0, 1):
        mc.autotune_reset()
        path = tmp_path / f"kc{v}.tsv"
        path.write_text(f"{keys[0]}\t{v}\t\n")
        mc.autotune_load(str(path))
        got.append(mc.kmeanspp(X, k, msr=msr, prior=prior, seed=5, weights=w))
        assert mc.autotune_report()["entries"][keys[0]]["variant"] == v
    for a, b in zip(got[0], got[1]):
        assert np.array_equal(a, b, equal_nan=True)
    if msr in (0, 2, 6) and n <= 20011:
        oids, oasn, ocosts = orc.kmeanspp(X, k, msr, prior, orc.uniforms(5, k), weights=w)
        assert np.array_equal(got[1][0], oids)
        assert np.array_equal(got[1][1], oasn)
        assert np.array_equal(got[1][2], ocosts.astype(got[1][2].dtype))
    if dup:
        assert len(set(X[got[1][0].astype(np.int64)].tobytes()[i * d * 4:(i + 1) * d * 4] for i in range(k))) == 5
    mc.autotune_reset()



@pytest.mark.parametrize("msr,prior,d", [(2, 0.0, 64), (5, 1.0, 36), (0, 0.5, 100)])
def test_kmeanspp_dense_update_variants_equal_oracle(mc, orc, msr, prior, d, tmp_path):
    """The dense k-means++ distance update in each form, forced through a loaded decision: rows
    staged per CTA (variant 0), read directly (1), or persistent CTAs streaming (tile, chunk)
    items across tile boundaries (2).  A matrix beyond the persistent-cluster sizes (n d >
    2^23), d with a partial last 32-column chunk; ids, assignments and costs equal the oracle's
    (SQRL2, L1) or each other (MKL)."""
    n = 150_000 if d <= 64 else 90_000
    rng = np.random.default_rng(d + msr)
    if msr == 5:
        X = rng.integers(0, 6, size=(n, d)).astype(np.float32)
    else:
        X = (rng.normal(size=(n, d)) * 2.0 + rng.integers(0, 8, size=(n, 1))).astype(np.float32)
    k = 12
    mc.autotune(True)
    mc.autotune_reset()
    mc.kmeanspp(X, k, msr=msr, prior=prior, seed=9)
    keys = [kk for kk in mc.autotune_report()["entries"] if kk.startswith(f"kmpp_dense|msr{msr}|")]
    assert len(keys) == 1 and len(mc.autotune_report()["entries"][keys[0]]["ms"]) == 3
    prune = [kk for kk in mc.autotune_report()["entries"] if kk.startswith("kmpp_prune|")]
    got = []
    for v in (0, 1, 2):
        mc.autotune_reset()
        path = tmp_path / f"upd{v}.tsv"
        lines = f"{keys[0]}\t{v}\t\n" + "".join(f"{p}\t0\t\n" for p in prune)
        path.write_text(lines)
        mc.autotune_load(str(path))
        got.append(mc.kmeanspp(X, k, msr=msr, prior=prior, seed=9))
        assert mc.autotune_report()["entries"][keys[0]]["variant"] == v
    for r in got[1:]:
        for a, b in zip(got[0], r):
            assert np.array_equal(a, b)
    if msr in (0, 2):
        oids, oasn, ocosts = orc.kmeanspp(X, k, msr, prior, orc.uniforms(9, k))
        assert np.array_equal(got[2][0], oids)
        assert np.array_equal(got[2][1].astype(np.uint32), oasn)
        assert np.array_equal(got[2][2], ocosts.astype(np.float32))
    mc.autotune_reset()
