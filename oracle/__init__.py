"""ORACLE — test infrastructure only.

ctypes front end of ``mc_oracle.cpp``: a CPU restatement of minicore's clustering hot path
(``include/minicore/dist/applicator.h:1632-1915``, ``optim/kmeans.h:49-215``,
``clustering/solve.h:98-285``, ``clustering/centroid.h:81-178,649-779``,
``coreset/coreset.h:340-699``).  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg may import this package, and only as the checker; the
product package ``minicore_gb300`` never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB = os.path.join(_BUILD, "liboracle.so")
_SRC = os.path.join(_HERE, "mc_oracle.cpp")

L1, L2, SQRL2, JSM, JSD, MKL, HELLINGER = 0, 1, 2, 3, 4, 5, 6
BFL, FL, LFKF, VX, LBK = 0, 1, 2, 3, 4


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-ffp-contract=off keeps float arithmetic unfused)."""
    os.makedirs(_BUILD, exist_ok=True)
    if not force and os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC):
        return _LIB
    tmp = _LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp, _SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB)
    return _LIB


class _Matrix(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("pad", ctypes.c_int32), ("n", ctypes.c_uint64),
                ("d", ctypes.c_uint64), ("vals", ctypes.c_void_p), ("idx", ctypes.c_void_p),
                ("indptr", ctypes.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P, U64, D, I = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, ctypes.c_int
        U32 = ctypes.c_uint32
        sig = {
            "orc_uniform": (D, [U64, U64]),
            "orc_uniforms": (None, [U64, U64, U64, P]),
            "orc_det_sum": (D, [P, U64]),
            "orc_det_draw": (U64, [P, U64, D]),
            "orc_msr_dense": (D, [I, P, P, U64, D, D, D, D]),
            "orc_msr_sparse": (D, [I, P, P, U64, P, P, U64, U64, D, D, D, D]),
            "orc_assign": (I, [P, P, U32, I, D, P, P]),
            "orc_kmeanspp": (I, [P, U32, I, D, P, P, P, P, P]),
            "orc_kmeanspp_greedy": (I, [P, U32, I, D, P, U32, U64, P, P, P]),
            "orc_lspp": (I, [P, U32, I, D, P, U64, U64, P, P, P]),
            "orc_hcluster": (I, [P, P, U32, I, D, P, D, U64, U64, P, P, P, P, P, P]),
            "orc_l1_centers": (I, [P, P, U32, P, P]),
            "orc_scluster": (I, [P, P, U32, I, D, P, D, U64, D, P, P, P, P, P, P]),
            "orc_minibatch": (I, [P, P, U32, I, D, P, U64, U64, U64, U64, I, U64, P, P, P, P, P, P]),
            "orc_sensitivity": (I, [U64, U64, U64, P, I, P, P, I, D, P]),
            "orc_alias_build": (I, [U64, P, P, P]),
            "orc_alias_draw": (U64, [U64, P, P, U64, U64]),
            "orc_coreset_sample": (None, [U64, P, P, P, P, I, U64, U64, U64, I, P, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Matrix:
    """Dense f32 (n x d) or CSR (f32 values, u32 indices, u64 indptr) view kept alive."""

    def __init__(self, X):
        import scipy.sparse as sp
        if sp.issparse(X):
            X = sp.csr_matrix(X)
            X.sort_indices()
            self.vals = np.ascontiguousarray(X.data, dtype=np.float32)
            self.idx = np.ascontiguousarray(X.indices, dtype=np.uint32)
            self.indptr = np.ascontiguousarray(X.indptr, dtype=np.uint64)
            self.n, self.d = X.shape
            self.kind = 1
        else:
            self.vals = np.ascontiguousarray(X, dtype=np.float32)
            self.idx = self.indptr = None
            self.n, self.d = self.vals.shape
            self.kind = 0
        self.s = _Matrix(self.kind, 0, self.n, self.d, self.vals.ctypes.data,
                         None if self.idx is None else self.idx.ctypes.data,
                         None if self.indptr is None else self.indptr.ctypes.data)

    def ref(self):
        return ctypes.byref(self.s)


def uniforms(seed: int, m: int, offset: int = 0) -> np.ndarray:
    out = np.empty(m, dtype=np.float64)
    lib().orc_uniforms(seed, offset, m, _p(out))
    return out


def det_sum(v) -> float:
    v = np.ascontiguousarray(v, dtype=np.float64)
    return lib().orc_det_sum(_p(v), v.size)


def det_draw(v, u: float) -> int:
    v = np.ascontiguousarray(v, dtype=np.float64)
    return int(lib().orc_det_draw(_p(v), v.size, u))


def msr_dense(msr, row, center, prior, prior_sum=None, rowsum=None, ctrsum=None):
    row = np.ascontiguousarray(row, dtype=np.float32)
    center = np.ascontiguousarray(center, dtype=np.float32)
    d = row.size
    prior_sum = prior * d if prior_sum is None else prior_sum
    rowsum = float(row.astype(np.float64).sum()) if rowsum is None else rowsum
    ctrsum = float(center.astype(np.float64).sum()) if ctrsum is None else ctrsum
    return lib().orc_msr_dense(msr, _p(row), _p(center), d, prior, prior_sum, rowsum, ctrsum)


def msr_sparse(msr, row, center, prior, prior_sum=None):
    """row/center: dense 1-D arrays converted to sparse (nonzero entries)."""
    row = np.asarray(row, dtype=np.float32)
    center = np.asarray(center, dtype=np.float32)
    d = row.size
    ri = np.nonzero(row)[0].astype(np.uint32)
    ci = np.nonzero(center)[0].astype(np.uint32)
    rv = np.ascontiguousarray(row[ri])
    cv = np.ascontiguousarray(center[ci])
    prior_sum = prior * d if prior_sum is None else prior_sum
    return lib().orc_msr_sparse(msr, _p(rv), _p(ri), ri.size, _p(cv), _p(ci), ci.size, d, prior,
                                prior_sum, float(row.astype(np.float64).sum()),
                                float(center.astype(np.float64).sum()))


def assign(X, centers, msr, prior):
    M = Matrix(X)
    C = np.ascontiguousarray(centers, dtype=np.float32)
    asn = np.empty(M.n, dtype=np.uint32)
    costs = np.empty(M.n, dtype=np.float64)
    lib().orc_assign(M.ref(), _p(C), C.shape[0], msr, prior, _p(asn), _p(costs))
    return asn, costs


def kmeanspp(X, k, msr, prior, uniforms_, weights=None):
    M = Matrix(X)
    u = np.ascontiguousarray(uniforms_, dtype=np.float64)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    kk = min(k, M.n)
    ids = np.empty(kk, dtype=np.uint32)
    asn = np.empty(M.n, dtype=np.uint32)
    costs = np.empty(M.n, dtype=np.float64)
    rc = lib().orc_kmeanspp(M.ref(), k, msr, prior, _p(w), _p(u), _p(ids), _p(asn), _p(costs))
    if rc:
        raise ValueError("orc_kmeanspp failed")
    return ids, asn, costs


def l1_centers(X, asn, k, weights=None):
    """The L1 center rule (set_centroids_l1's medians) for a given assignment, dense or CSR
    rows (no empty cluster)."""
    M = Matrix(X)
    a = np.ascontiguousarray(asn, dtype=np.uint32)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    out = np.empty((k, M.d), np.float32)
    rc = lib().orc_l1_centers(M.ref(), _p(a), k, _p(w), _p(out))
    if rc:
        raise ValueError(f"orc_l1_centers failed ({rc})")
    return out


def kmeanspp_greedy(X, k, msr, prior, n_local_trials, seed, weights=None):
    M = Matrix(X)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    kk = min(k, M.n)
    ids = np.empty(kk, dtype=np.uint32)
    asn = np.empty(M.n, dtype=np.uint32)
    costs = np.empty(M.n, dtype=np.float64)
    rc = lib().orc_kmeanspp_greedy(M.ref(), k, msr, prior, _p(w), n_local_trials, seed, _p(ids), _p(asn), _p(costs))
    if rc:
        raise ValueError("orc_kmeanspp_greedy failed")
    return ids, asn, costs


def lspp(X, ids, msr, prior, rounds, seed, weights=None):
    """localsearch++ rounds on seeded center ids (returns ids, asn, costs)."""
    M = Matrix(X)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    ids = np.array(ids, dtype=np.uint32, copy=True)
    asn = np.empty(M.n, dtype=np.uint32)
    costs = np.empty(M.n, dtype=np.float64)
    rc = lib().orc_lspp(M.ref(), ids.size, msr, prior, _p(w), rounds, seed, _p(ids), _p(asn), _p(costs))
    if rc:
        raise ValueError("orc_lspp failed")
    return ids, asn, costs


def hcluster(X, centers, msr, prior, weights=None, eps=1e-10, maxiter=100, seed=1):
    M = Matrix(X)
    C = np.ascontiguousarray(centers, dtype=np.float32)
    k = C.shape[0]
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    cout = np.empty_like(C)
    asn = np.empty(M.n, dtype=np.uint32)
    costs = np.empty(M.n, dtype=np.float64)
    ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
    rc = lib().orc_hcluster(M.ref(), _p(C), k, msr, prior, _p(w), eps, maxiter, seed, _p(cout), _p(asn),
                            _p(costs), ctypes.byref(ic), ctypes.byref(fc), ctypes.byref(it))
    if rc == 2:
        raise RuntimeError("Unexpected nan in ctr")
    if rc == 3:
        raise NotImplementedError("Not implemented: weighted L1 median for CSparseMatrix")
    return dict(initcost=ic.value, finalcost=fc.value, numiter=it.value, centers=cout, asn=asn,
                costs=costs)


def minibatch(X, centers, msr, prior, weights=None, mbsize=100, maxiter=20, freq=5, reseed_after=1,
              with_rep=False, seed=1):
    M = Matrix(X)
    C = np.ascontiguousarray(centers, dtype=np.float32)
    k = C.shape[0]
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    cout = np.empty_like(C)
    asn = np.empty(M.n, dtype=np.uint32)
    costs = np.empty(M.n, dtype=np.float64)
    ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
    rc = lib().orc_minibatch(M.ref(), _p(C), k, msr, prior, _p(w), mbsize, maxiter, freq, reseed_after,
                             int(bool(with_rep)), seed, _p(cout), _p(asn), _p(costs), ctypes.byref(ic),
                             ctypes.byref(fc), ctypes.byref(it))
    if rc == 2:
        raise RuntimeError("Unexpected nan in ctr")
    if rc == 3:
        raise NotImplementedError("Not implemented: weighted L1 median for CSparseMatrix")
    return dict(initcost=ic.value, finalcost=fc.value, numiter=it.value, centers=cout, asn=asn, costs=costs)


def scluster(X, centers, msr, prior, weights=None, temp=1.0, maxiter=1000, eps=1e-8):
    M = Matrix(X)
    C = np.ascontiguousarray(centers, dtype=np.float32)
    k = C.shape[0]
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    cout = np.empty_like(C)
    costs = np.empty((M.n, k), dtype=np.float32)
    asn = np.empty((M.n, k), dtype=np.float32)
    ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
    rc = lib().orc_scluster(M.ref(), _p(C), k, msr, prior, _p(w), temp, maxiter, eps, _p(cout), _p(costs),
                            _p(asn), ctypes.byref(ic), ctypes.byref(fc), ctypes.byref(it))
    if rc:
        raise ValueError("orc_scluster failed")
    return dict(initcost=ic.value, finalcost=fc.value, numiter=it.value, centers=cout, costs=costs, asn=asn)


def sensitivity(costs, asn, ncenters, method, weights=None, k=None, alpha_est=0.0):
    costs = np.ascontiguousarray(costs)
    f64 = 1 if costs.dtype == np.float64 else 0
    if not f64:
        costs = costs.astype(np.float32)
    asn = np.ascontiguousarray(asn, dtype=np.uint32)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
    probs = np.empty(costs.size, dtype=np.float32)
    rc = lib().orc_sensitivity(costs.size, ncenters, ncenters if k is None else k, _p(costs), f64, _p(asn),
                               _p(w), method, alpha_est, _p(probs))
    if rc:
        raise ValueError("orc_sensitivity failed")
    return probs


def alias_build(probs):
    probs = np.ascontiguousarray(probs, dtype=np.float32)
    pt = np.empty(probs.size, dtype=np.float64)
    at = np.empty(probs.size, dtype=np.uint32)
    if lib().orc_alias_build(probs.size, _p(probs), _p(pt), _p(at)):
        raise ValueError("alias build failed")
    return pt, at


def coreset_sample(probs, prob_tab, alias_tab, m, seed, unique=False, weights=None, method=0, b=0):
    probs = np.ascontiguousarray(probs, dtype=np.float32)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
    wo = np.empty(m, dtype=np.float32)
    io = np.empty(m, dtype=np.uint64)
    lib().orc_coreset_sample(probs.size, _p(probs), _p(prob_tab), _p(alias_tab), _p(w), method, b, m, seed,
                             int(bool(unique)), _p(wo), _p(io))
    return wo, io


def coreset_minibatch(X, centers, msr, prior, mbsize, maxiter, ncheckins=10, reseed_count=5, seed=0, weights=None):
    """Minibatch-by-coreset EM (hmb_coreset_clustering, clustering/solve.h:593-789, as called
    by python/pycluster.h:36-38), restated over the oracle's pieces with the canonical
    randomness of the device path: restarts draw U(seed, r) over costs (x row weights), the
    coreset sample seed is floor(U(seed, r) * 2^53), one counter r for both, in order; the
    coreset sub-clustering is perform_hard_clustering with eps 1e-3, 1 update (3 in the first
    two rounds) and restart seed = coreset size.  Returns (best centers, asn, costs of the last
    exhaustive assignment, initcost, bestcost, rounds)."""
    import scipy.sparse as sp
    C = np.array(centers, dtype=np.float32, copy=True)
    k = C.shape[0]
    n = X.shape[0]
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    freq = (maxiter + ncheckins - 1) // ncheckins
    rounds = (freq - 1 + maxiter) // freq
    m = min(max(int(mbsize), 1), n)
    alpha = 1.0 if msr == 0 else 2.0 if msr == 2 else 4.0
    method = 3 if msr == 0 else 4            # VX for L1, else LBK
    counter = 0
    best = C.copy()
    initcost = bestcost = 0.0
    it = 0
    dense_row = (lambda i: np.asarray(X[i].toarray(), np.float32).ravel()) if sp.issparse(X) else (lambda i: X[i])
    while True:
        asn, costs = assign(X, C, msr, prior)
        cnt = np.bincount(asn, minlength=k)
        found = [c for c in range(k) if cnt[c] <= reseed_count]
        if found:
            for f in found:
                u = float(uniforms(seed, 1, offset=counter)[0])
                counter += 1
                r = det_draw(costs * w if w is not None else costs, u)
                C[f] = dense_row(r if r < n else 0)
            a2, c2 = assign(X, C[found], msr, prior)
            better = c2 < costs
            asn = np.where(better, np.asarray(found, np.uint32)[a2], asn).astype(np.uint32)
            costs = np.where(better, c2, costs)
        cost = det_sum(costs * w if w is not None else costs)
        if it == 0:
            initcost = bestcost = cost
        elif cost < bestcost:
            bestcost = cost
            best = C.copy()
        it += 1
        if it > rounds:
            break
        probs = sensitivity(costs, asn, k, method, weights=w, k=k, alpha_est=alpha)
        pt, at = alias_build(probs)
        for _ in range(freq):
            sseed = int(float(uniforms(seed, 1, offset=counter)[0]) * 9007199254740992.0)
            counter += 1
            wo, io = coreset_sample(probs, pt, at, m, sseed, unique=True, weights=w, method=method, b=k)
            io = io.astype(np.int64)
            cw = wo.astype(np.float64) * (w[io] if w is not None else 1.0)
            sub = hcluster(X[io], C, msr, prior, weights=cw, eps=1e-3, maxiter=1 + (2 if it < 2 else 0), seed=m)
            C = np.asarray(sub["centers"], np.float32)
    return best, asn, costs, initcost, bestcost, it
