"""minicore_gb300 — GB300-native clustering hot path with minicore's Python entry points.

Drop-in functions (same names, argument meanings and defaults as the reference's
``minicore`` package, ``minicore/__init__.py:23-163`` and the pybind11 module
``pyminicore``):

* ``kmeanspp(matrix, k, *, msr=2, prior=0., seed=0, ntimes=1, lspp=0, expskips=0,
  n_local_trials=1, weights=None)`` -> ``(center_ids u32[k], asn u8/u16/u32[n], costs)``
  (``python/pydense.cpp:34-77``, ``python/smw.h:179-412``);
* ``hcluster(matrix, centers, *, prior=0., msr=2, weights=None, eps=1e-10, maxiter=1000,
  ...)`` -> ``{initcost, finalcost, numiter, centers, costs, asn}``
  (``python/pycluster_dense.cpp:69-112``, ``python/pycluster.h:10-205``);
* ``CoresetSampler`` with ``make_sampler / get_probs / sample`` (``python/pycs.cpp:3-58``);
* ``CSparseMatrix`` (``python/pycsparse.cpp:15-89``) and ``cluster`` (``minicore/__init__.py:235-261``).

All computation runs in the CUDA library ``libminicore_gb300.so`` through its C ABI
(``include/minicore_gb300.h``).  There is no CPU fallback.

Differences from the reference, by design:
* randomness: the reference's wy/aesctr RNG streams and libsimdsampling are not part of
  its tree; every draw here consumes U(seed, i) of a splitmix64 stream (``uniforms``);
* float64 inputs are computed in float32 (the reference computes them in float64);
* ``precision="bf16"|"tf32"`` selects the tensor-core SQRL2 assignment for dense data.
"""
from __future__ import annotations

import ctypes
import gzip
import os
import struct
import threading

import numpy as np

from . import _lib
from ._lib import McError, McMatrix, check

__all__ = ["kmeanspp", "hcluster", "cluster", "CoresetSampler", "CSparseMatrix", "Context", "Job",
           "uniforms", "library_path", "L1", "SQRL2", "JSD", "MKL", "HELLINGER",
           "BFL", "FL", "LFKF", "VX", "LBK"]

L1, SQRL2, JSD, MKL, HELLINGER = 0, 2, 4, 5, 6
BFL, FL, LFKF, VX, LBK = 0, 1, 2, 3, 4
_MEASURE_NAMES = {"L1": 0, "SQRL2": 2, "JSD": 4, "MKL": 5, "HELLINGER": 6}
_PREC = {"fp32": _lib.MC_FP32, "tf32": _lib.MC_TF32, "bf16": _lib.MC_BF16}

library_path = _lib.library_path


def _msr(m) -> int:
    if isinstance(m, str):
        key = m.upper()
        if key not in _MEASURE_NAMES:
            raise NotImplementedError(f"measure {m!r} is outside the implemented hot path")
        return _MEASURE_NAMES[key]
    return int(m)


def _p(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def _seed(seed) -> int:
    seed = int(seed)
    if seed == 0:  # the reference draws a random seed for 0 (python/smw.h:188)
        seed = int.from_bytes(os.urandom(8), "little") or 1
    return seed & 0xFFFFFFFFFFFFFFFF


def uniforms(seed: int, m: int, offset: int = 0) -> np.ndarray:
    """U(seed, offset + i), i < m: the splitmix64 stream every draw of this library uses."""
    out = np.empty(m, dtype=np.float64)
    check(_lib.load().mc_uniforms(seed, offset, m, _p(out)))
    return out


# ------------------------------------------------------------------------------------
# context
# ------------------------------------------------------------------------------------
class Context:
    """One CUDA device + stream.  Thread-compatible; one per thread for concurrency."""

    def __init__(self, device: int = 0):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.mc_context_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device

    def set_stream(self, stream_ptr: int | None):
        check(self._lib.mc_context_set_stream(self.handle, ctypes.c_void_p(stream_ptr or 0)))

    def synchronize(self):
        check(self._lib.mc_context_synchronize(self.handle))

    def close(self):
        if getattr(self, "handle", None):
            self._lib.mc_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def default_context() -> Context:
    ctx = getattr(_tls, "ctx", None)
    if ctx is None:
        ctx = Context(0)
        _tls.ctx = ctx
    return ctx


# ------------------------------------------------------------------------------------
# matrices
# ------------------------------------------------------------------------------------
class CSparseMatrix:
    """Zero-copy view of CSR arrays (python/pycsparse.h:33-70).  Values are used as float32,
    column indices as uint32 and row offsets as uint64; other dtypes are converted once."""

    def __init__(self, sparray=None, *, data=None, indices=None, indptr=None, shape=None):
        if sparray is not None:
            if isinstance(sparray, tuple) and len(sparray) == 2 and isinstance(sparray[0], tuple):
                (data, indices, indptr), shape = sparray
            else:
                data, indices, indptr = sparray.data, sparray.indices, sparray.indptr
                shape = sparray.shape
        self.data = data if (hasattr(data, "data_ptr") or (isinstance(data, np.ndarray) and data.dtype == np.float32
                                                             and data.flags.c_contiguous)) \
            else np.ascontiguousarray(data, dtype=np.float32)
        self.indices = indices if (hasattr(indices, "data_ptr") or (isinstance(indices, np.ndarray)
                                   and indices.dtype == np.uint32 and indices.flags.c_contiguous)) \
            else np.ascontiguousarray(indices, dtype=np.uint32)
        self.indptr = indptr if (hasattr(indptr, "data_ptr") or (isinstance(indptr, np.ndarray)
                                 and indptr.dtype == np.uint64 and indptr.flags.c_contiguous)) \
            else np.ascontiguousarray(indptr, dtype=np.uint64)
        self.shape = (int(shape[0]), int(shape[1]))

    @staticmethod
    def from_items(data, indices, indptr, shape):
        return CSparseMatrix(data=data, indices=indices, indptr=indptr, shape=shape)

    def rows(self):
        return self.shape[0]

    def columns(self):
        return self.shape[1]

    def nnz(self):
        return int(self.data.shape[0]) if hasattr(self.data, "shape") else len(self.data)

    def __str__(self):
        return f"CSparseMatrix, {self.shape[0]}x{self.shape[1]}, {self.nnz()}"


def _is_sparse(x) -> bool:
    try:
        import scipy.sparse as sp
        if sp.issparse(x):
            return True
    except ImportError:  # pragma: no cover
        pass
    return isinstance(x, CSparseMatrix)


class _MatrixArg:
    """Keeps the arrays behind an mc_matrix alive for the duration of a call."""

    def __init__(self, X):
        if _is_sparse(X):
            if not isinstance(X, CSparseMatrix):
                import scipy.sparse as sp
                X = sp.csr_matrix(X)
                if not X.has_sorted_indices:
                    X = X.sorted_indices()
                X = CSparseMatrix(X)
            self.keep = X
            self.kind = _lib.MC_CSR_F32
            self.n, self.d = X.shape
            self.m = McMatrix(_lib.MC_CSR_F32, 0, self.n, self.d, _p(X.data), _p(X.indices), _p(X.indptr),
                              X.nnz())
        else:
            if hasattr(X, "data_ptr"):  # torch tensor (device-resident input)
                if X.dtype.__str__() != "torch.float32" or not X.is_contiguous() or X.dim() != 2:
                    raise ValueError("device matrices must be contiguous 2-D float32 tensors")
                self.keep = X
                self.n, self.d = X.shape
            else:
                A = np.ascontiguousarray(X, dtype=np.float32)
                if A.ndim != 2:
                    raise ValueError("Wrong number of dimensions")
                self.keep = A
                self.n, self.d = A.shape
            self.kind = _lib.MC_DENSE_F32
            self.m = McMatrix(_lib.MC_DENSE_F32, 0, self.n, self.d, _p(self.keep), None, None, 0)

    @property
    def ref(self):
        return ctypes.byref(self.m)


def _row_dense(M: _MatrixArg, r: int) -> np.ndarray:
    X = M.keep
    if M.kind == _lib.MC_DENSE_F32:
        return np.asarray(X[r], dtype=np.float32) if not hasattr(X, "data_ptr") else X[r].cpu().numpy()
    out = np.zeros(M.d, dtype=np.float32)
    ip = np.asarray(X.indptr)
    b, e = int(ip[r]), int(ip[r + 1])
    out[np.asarray(X.indices)[b:e].astype(np.int64)] = np.asarray(X.data)[b:e]
    return out


def _centers_array(M: _MatrixArg, centers) -> np.ndarray:
    """Center specification as in obj2dvec (python/pyhelpers.h:123-218): 1-D integer array or
    sequence of row ids, a 2-D array, or a sequence of 1-D arrays."""
    if isinstance(centers, np.ndarray) and centers.ndim == 2:
        C = np.ascontiguousarray(centers, dtype=np.float32)
    elif isinstance(centers, np.ndarray) and centers.ndim == 1 and np.issubdtype(centers.dtype, np.integer):
        C = np.stack([_row_dense(M, int(r)) for r in centers])
    elif isinstance(centers, (list, tuple)) and len(centers) and isinstance(centers[0], np.ndarray):
        C = np.stack([np.asarray(c, dtype=np.float32).ravel() for c in centers])
    elif isinstance(centers, (list, tuple)):
        C = np.stack([_row_dense(M, int(r)) for r in centers])
    else:
        raise ValueError("Invalid: expected numpy array or list of numpy arrays or list of center ids")
    if C.ndim != 2 or C.shape[1] != M.d:
        raise ValueError("centers must have as many columns as the matrix")
    return np.ascontiguousarray(C, dtype=np.float32)


# ------------------------------------------------------------------------------------
# kmeans++
# ------------------------------------------------------------------------------------
def _asn_dtype(k: int):
    # python/smw.h:329-341 (dense) and 211-220 (CSR)
    if k <= 256:
        return np.uint8
    if k <= 63356:
        return np.uint16
    return np.uint32


def kmeanspp(matrix, k, *, msr=2, prior=0., seed=0, ntimes=1, lspp=0, expskips=0, n_local_trials=1,
             weights=None, ctx: Context | None = None):
    """D^2 seeding (include/minicore/optim/kmeans.h:49-215).  Returns (center ids,
    assignments, costs); costs are float32 for dense input and float64 for CSR input, as in
    the reference bindings.  ``n_local_trials > 1``: greedy seeding (mc_kmeanspp_greedy, uniforms
    U(seed + run, r)); ``lspp`` > 0: that many localsearch++ rounds afterwards (mc_kmeanspp_ex)."""
    trials = max(int(n_local_trials or 1), 1)
    lspp = max(int(lspp or 0), 0)
    ctx = ctx or default_context()
    M = _MatrixArg(matrix)
    k = int(k)
    if k <= 0:
        raise ValueError("k must be positive")
    if prior < 0:
        prior = 1.0 / M.d  # python/smw.h:184-187
    seed = _seed(seed)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    kk = min(k, M.n)
    # dense: ntimes - 1 extra runs, best total cost kept (python/pydense.cpp:41, smw.h:385-393).
    # CSR: the reference compares the extra runs against the first run's own cost
    # (python/smw.h:250), so the first run is always returned.
    runs = max(int(ntimes), 1) if M.kind == _lib.MC_DENSE_F32 else 1
    best = None
    for t in range(runs):
        ids = np.empty(kk, dtype=np.uint32)
        asn = np.empty(M.n, dtype=np.uint32)
        costs = np.empty(M.n, dtype=np.float64)
        if lspp:
            check(_lib.load().mc_kmeanspp_ex(ctx.handle, M.ref, k, _msr(msr), float(prior), _p(w), trials, lspp,
                                             (seed + t) & 0xFFFFFFFFFFFFFFFF, _p(ids), _p(asn), _p(costs)))
        elif trials > 1:
            check(_lib.load().mc_kmeanspp_greedy(ctx.handle, M.ref, k, _msr(msr), float(prior), _p(w), trials,
                                                 (seed + t) & 0xFFFFFFFFFFFFFFFF, _p(ids), _p(asn), _p(costs)))
        else:
            u = uniforms(seed, k, offset=t * k)
            check(_lib.load().mc_kmeanspp(ctx.handle, M.ref, k, _msr(msr), float(prior), _p(w), _p(u), _p(ids),
                                          _p(asn), _p(costs)))
        c = costs.sum()
        if best is None or c < best[0]:
            best = (c, ids, asn, costs)
    _, ids, asn, costs = best
    asn = asn.astype(_asn_dtype(k))
    if M.kind == _lib.MC_DENSE_F32:
        costs = costs.astype(np.float32)
    return ids, asn, costs


# ------------------------------------------------------------------------------------
# hcluster
# ------------------------------------------------------------------------------------
def _centers_to_csr(C: np.ndarray):
    """centers2pylist (python/pyhelpers.h:67-112): ((data f32, idx u32, indptr u64), shape)."""
    nz = C != 0
    indptr = np.zeros(C.shape[0] + 1, dtype=np.uint64)
    indptr[1:] = np.cumsum(nz.sum(1))
    rows, cols = np.nonzero(nz)
    return ((C[rows, cols].astype(np.float32), cols.astype(np.uint32), indptr),
            np.array(C.shape, dtype=np.uint64))


def hcluster(matrix, centers, *, prior=0., msr=2, weights=None, eps=1e-10, maxiter=1000, mbsize=-1,
             ncheckins=-1, with_rep=False, cs=False, seed=0, reseed_count=5, precision="fp32",
             ctx: Context | None = None):
    """Hard Lloyd/Bregman EM from explicit centers (clustering/solve.h:98-175); with
    mbsize >= 0, minibatch EM (solve.h:386-582) with maxiter iterations, a check-in every
    ceil(maxiter / ncheckins), restarts of centers holding <= reseed_count rows, and
    with_rep sampling; with cs=True as well, minibatch-by-coreset EM (hmb_coreset_clustering,
    solve.h:593-789)."""
    ctx = ctx or default_context()
    M = _MatrixArg(matrix)
    C = _centers_array(M, centers)
    k = C.shape[0]
    if prior < 0:
        prior = 1.0 / M.d
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    cout = np.empty_like(C)
    asn = np.empty(M.n, dtype=np.uint32)
    ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
    if mbsize is not None and int(mbsize) >= 0:
        costs = np.empty(M.n, dtype=np.float64)
        # perform_hard_minibatch_clustering (python/pycluster.h:31-40): ncheckins < 0 -> 10
        nchk = int(ncheckins) if ncheckins is not None and int(ncheckins) > 0 else 10
        if cs:  # pycluster.h:36-38
            check(_lib.load().mc_hcluster_coreset(ctx.handle, M.ref, _p(C), k, _msr(msr), float(prior), _p(w),
                                                  max(int(mbsize), 1), int(maxiter), nchk, int(reseed_count),
                                                  _seed(seed), _PREC[precision], _p(cout), _p(asn), _p(costs),
                                                  ctypes.byref(ic), ctypes.byref(fc), ctypes.byref(it)))
        else:
            check(_lib.load().mc_hcluster_minibatch(ctx.handle, M.ref, _p(C), k, _msr(msr), float(prior), _p(w),
                                                    max(int(mbsize), 1), int(maxiter), nchk, int(reseed_count),
                                                    int(bool(with_rep)), _seed(seed), _PREC[precision], _p(cout),
                                                    _p(asn), _p(costs), ctypes.byref(ic), ctypes.byref(fc),
                                                    ctypes.byref(it)))
    else:
        # the costs come back as float32, rounded on the device (python/pycluster.h:59)
        costs = np.empty(M.n, dtype=np.float32)
        check(_lib.load().mc_hcluster_f32(ctx.handle, M.ref, _p(C), k, _msr(msr), float(prior), _p(w), float(eps),
                                          int(maxiter), _seed(seed), _PREC[precision], _p(cout), _p(asn), _p(costs),
                                          ctypes.byref(ic), ctypes.byref(fc), ctypes.byref(it)))
    centers_out = cout if M.kind == _lib.MC_DENSE_F32 else _centers_to_csr(cout)
    return {"initcost": ic.value, "finalcost": fc.value, "numiter": it.value, "centers": centers_out,
            "costs": costs if costs.dtype == np.float32 else costs.astype(np.float32), "asn": asn}


def scluster(matrix, centers, msr=2, prior=0., temp=1., maxiter=1000, mbsize=-1, mbn=-1, savepref="",
             weights=None, ctx: Context | None = None):
    """Soft clustering from explicit centers (perform_soft_clustering, clustering/solve.h:287-374;
    python/pycluster_softdense.cpp:66-90).  Returns initcost, finalcost, numiter, centers, and
    the last (rows x k) float32 cost and soft-assignment matrices; eps 1e-8.  CSR rows give CSR
    centers, as hcluster does."""
    if mbsize is not None and int(mbsize) > 0:
        raise NotImplementedError("Not yet completed: minibatch soft clustering")
    ctx = ctx or default_context()
    M = _MatrixArg(matrix)
    C = _centers_array(M, centers)
    k = C.shape[0]
    if prior < 0:
        prior = 0.
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    cout = np.empty_like(C)
    costs = np.empty((M.n, k), dtype=np.float32)
    asn = np.empty((M.n, k), dtype=np.float32)
    ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
    check(_lib.load().mc_scluster(ctx.handle, M.ref, _p(C), k, _msr(msr), float(prior), _p(w), float(temp),
                                  int(maxiter), 1e-8, _p(cout), _p(costs), _p(asn), ctypes.byref(ic),
                                  ctypes.byref(fc), ctypes.byref(it)))
    centers_out = cout if M.kind == _lib.MC_DENSE_F32 else _centers_to_csr(cout)
    return {"initcost": ic.value, "finalcost": fc.value, "numiter": it.value, "centers": centers_out,
            "costs": costs, "asn": asn}


def cluster_from_centers(*args, **kwargs):
    return hcluster(*args, **kwargs)


def cluster(data, *, msr, k, prior=0., seed=0, nmkc=0, ntimes=1, lspp=0, use_exponential_skips=False,
            n_local_trials=1, weights=None, mbsize=-1, clustereps=1e-4, temp=-1., cs=False, with_rep=True,
            outpref="mc.cluster.output", maxiter=50, precision="fp32"):
    """kmeans++ then hcluster, or scluster when temp > 0 (minicore/__init__.py:235-261)."""
    seed = _seed(seed)
    ids, asn, costs = kmeanspp(data, k, msr=msr, prior=prior, seed=seed, ntimes=ntimes, lspp=lspp,
                               n_local_trials=n_local_trials, weights=weights)
    if temp > 0:
        return scluster(data, ids.astype(np.int64), msr=msr, prior=prior, temp=temp, maxiter=maxiter,
                        weights=weights)
    return hcluster(data, ids.astype(np.int64), prior=prior, msr=msr, weights=weights, eps=clustereps,
                    maxiter=maxiter, seed=seed, precision=precision)


# ------------------------------------------------------------------------------------
# pairwise distances
# ------------------------------------------------------------------------------------
def cmp(matrix, data, msr=2, prior=0., reverse=None, use_float=-1, ctx: Context | None = None):
    """Distances between the rows of ``matrix`` and the rows of ``data`` (python/pycmp.cpp:15-246,
    python/pyarrcmp.cpp:52-144), float32, shape (rows of matrix, rows of data).

    Default roles are the assignment's: out[i, j] = msr(lh = data[j], rh = matrix[i]).  As in
    the reference, ``reverse`` flips them with opposite defaults per overload: for a NumPy
    ``matrix`` reverse=True (its default) keeps those roles, for a sparse ``matrix``
    reverse=False (its default) keeps them.  1-D ``data`` gives one value per row of
    ``matrix``; 1-D ``matrix`` and ``data`` give a float."""
    ctx = ctx or default_context()
    scalar = False
    if not _is_sparse(matrix) and not hasattr(matrix, "data_ptr"):
        matrix = np.asarray(matrix)
        if matrix.ndim == 1:
            matrix = matrix[None, :]
            scalar = True
    M = _MatrixArg(matrix)
    if _is_sparse(data):
        data = data.toarray() if hasattr(data, "toarray") else np.asarray(data)
    Y = np.asarray(data, dtype=np.float32)
    one = Y.ndim == 1
    if one:
        Y = Y[None, :]
    if Y.ndim != 2:
        raise ValueError("NumPy array expected to have 1 or two dimensions.")
    if Y.shape[1] != M.d:
        raise ValueError("Array must be of the same dimensionality as the matrix")
    Y = np.ascontiguousarray(Y)
    if reverse is None:
        assign_roles = True
    elif M.kind == _lib.MC_DENSE_F32:
        assign_roles = bool(reverse)
    else:
        assign_roles = not bool(reverse)
    out = np.empty((M.n, Y.shape[0]), dtype=np.float32)
    check(_lib.load().mc_cmp(ctx.handle, M.ref, _p(Y), Y.shape[0], _msr(msr), float(prior),
                             0 if assign_roles else 1, _p(out)))
    if scalar and one:
        return float(out[0, 0])
    return out[:, 0] if one else out


def pcmp(matrix, msr=2, prior=0., use_float=-1, ctx: Context | None = None):
    """Condensed pairwise distances among the rows of ``matrix`` (python/pycmp.cpp:249-300):
    entry i*n - i*(i+1)/2 + j - i - 1 = msr(lh = row i, rh = row j) for i < j, float32."""
    ctx = ctx or default_context()
    M = _MatrixArg(matrix)
    n = M.n
    out = np.empty(max(n * (n - 1) // 2, 0), dtype=np.float32)
    if n >= 2:
        check(_lib.load().mc_pcmp(ctx.handle, M.ref, _msr(msr), float(prior), _p(out)))
    return out


# ------------------------------------------------------------------------------------
# coreset sampler
# ------------------------------------------------------------------------------------
class CoresetSampler:
    """CoresetSampler<float, uint32_t> (include/minicore/coreset/coreset.h:228-701)."""

    def __init__(self, ctx: Context | None = None):
        self._ctx = ctx or default_context()
        self._h = None
        self.np_ = 0

    def make_sampler(self, ncenters, costs, assignments, weights=None, seed=13, sens=0):
        costs = np.asarray(costs)
        if costs.ndim != 1:
            raise ValueError("costs must be 1-dimensional")
        if costs.dtype == np.float64:
            c, f64 = np.ascontiguousarray(costs), 1
        elif costs.dtype == np.float32:
            c, f64 = np.ascontiguousarray(costs), 0
        else:
            raise ValueError("Costs is not double or float")
        a = np.ascontiguousarray(assignments, dtype=np.uint32)
        w = None
        if weights is not None:
            wa = np.asarray(weights)
            if wa.ndim != 1:
                raise ValueError("weightss must be 1-dimensional")
            if wa.dtype not in (np.float32, np.float64):
                raise ValueError("Weights can only be double or float")
            w = np.ascontiguousarray(wa, dtype=np.float32)
        self._release()
        h = ctypes.c_void_p()
        check(_lib.load().mc_sampler_create(self._ctx.handle, c.size, int(ncenters), int(ncenters), _p(c), f64,
                                            _p(a), _p(w), int(sens), 0.0, ctypes.byref(h)))
        self._h = h
        self.np_ = c.size
        self.seed_ = int(seed)
        self.sens_ = int(sens)
        return None

    def get_probs(self):
        out = np.empty(self.np_, dtype=np.float32)
        check(_lib.load().mc_sampler_probs(self._h, _p(out)))
        return out

    def alias_table(self):
        pt = np.empty(self.np_, dtype=np.float64)
        at = np.empty(self.np_, dtype=np.uint32)
        check(_lib.load().mc_sampler_alias(self._h, _p(pt), _p(at)))
        return pt, at

    def sample(self, size, seed=0, unique=False, eps=0.1):
        if self._h is None:
            raise ValueError("Can't sample without created sampler. Call make_ampler")
        size = int(size)
        wo = np.empty(size, dtype=np.float32)
        io = np.empty(size, dtype=np.uint64)
        check(_lib.load().mc_sampler_sample(self._h, size, _seed(seed), int(bool(unique)), _p(wo), _p(io)))
        return wo, io

    # ---- on-disk form (coreset.h:279-338): uint64 n, uint64 seed, float32 probs[n],
    # uint32 137 (weights follow: float32[n]) or 0.  Written gzip-compressed as the
    # reference's path-based write does (gzopen); read from gzip or plain files.
    def write(self, path):
        if self._h is None:
            raise ValueError("no sampler to write")
        if getattr(self, "sens_", 0) == FL:
            raise RuntimeError("Not implemented: serialization for FL coreset samplers")
        lib = _lib.load()
        probs = self.get_probs()
        hw = ctypes.c_int()
        check(lib.mc_sampler_info(self._h, None, None, ctypes.byref(hw)))
        parts = [struct.pack("<QQ", self.np_, getattr(self, "seed_", 137) & 0xFFFFFFFFFFFFFFFF), probs.tobytes()]
        if hw.value:
            w = np.empty(self.np_, dtype=np.float32)
            check(lib.mc_sampler_weights(self._h, _p(w)))
            parts += [struct.pack("<I", 137), w.tobytes()]
        else:
            parts.append(struct.pack("<I", 0))
        with gzip.open(path, "wb") as f:
            f.write(b"".join(parts))

    def read(self, path):
        raw = _read_maybe_gz(path)
        if len(raw) < 20:
            raise RuntimeError("Failed to read from file")
        n, seed = struct.unpack_from("<QQ", raw, 0)
        off = 16
        if len(raw) < off + 4 * n + 4:
            raise RuntimeError("Failed to read from file")
        probs = np.frombuffer(raw, dtype=np.float32, count=n, offset=off).copy()
        off += 4 * n
        (present,) = struct.unpack_from("<I", raw, off)
        off += 4
        w = None
        if present:
            if present != 137 or len(raw) < off + 4 * n:
                raise RuntimeError("Failed to read from file")
            w = np.frombuffer(raw, dtype=np.float32, count=n, offset=off).copy()
        self._release()
        h = ctypes.c_void_p()
        check(_lib.load().mc_sampler_from_probs(self._ctx.handle, n, _p(probs), _p(w), ctypes.byref(h)))
        self._h = h
        self.np_ = int(n)
        self.seed_ = int(seed)
        self.sens_ = BFL
        return self

    def _release(self):
        if self._h is not None:
            _lib.load().mc_sampler_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass


def _read_maybe_gz(path) -> bytes:
    with open(path, "rb") as f:
        head = f.read(2)
    if head == b"\x1f\x8b":
        with gzip.open(path, "rb") as f:
            return f.read()
    with open(path, "rb") as f:
        return f.read()


class IndexCoreset:
    """Indices and weights of a sampled coreset (IndexCoreset<IT, FT>,
    include/minicore/coreset/coreset.h:79-178).  On disk: uint64 size, IT indices[size],
    FT weights[size] (written gzip-compressed; read from gzip or plain files)."""

    def __init__(self, indices=None, weights=None, itype=np.uint32, ftype=np.float32):
        self.itype, self.ftype = np.dtype(itype), np.dtype(ftype)
        self.indices = np.asarray([] if indices is None else indices).astype(self.itype)
        self.weights = np.asarray([] if weights is None else weights).astype(self.ftype)
        if self.indices.shape != self.weights.shape:
            raise ValueError("indices and weights differ in length")

    def size(self):
        return int(self.indices.size)

    def write(self, path):
        with gzip.open(path, "wb") as f:
            f.write(struct.pack("<Q", self.size()) + self.indices.tobytes() + self.weights.tobytes())

    def read(self, path):
        raw = _read_maybe_gz(path)
        if len(raw) < 8:
            raise RuntimeError("Failed to read from file")
        (n,) = struct.unpack_from("<Q", raw, 0)
        ib, fb = self.itype.itemsize * n, self.ftype.itemsize * n
        if len(raw) < 8 + ib + fb:
            raise RuntimeError("Failed to read from file")
        self.indices = np.frombuffer(raw, dtype=self.itype, count=n, offset=8).copy()
        self.weights = np.frombuffer(raw, dtype=self.ftype, count=n, offset=8 + ib).copy()
        return self

    def compact(self):
        """Merge repeated (index, weight) pairs into one entry of weight count * weight,
        ordered by (index, weight); unchanged when every pair is distinct (coreset.h:138-163)."""
        pairs = {}
        for i, w in zip(self.indices.tolist(), self.weights.tolist()):
            key = (i, w)
            pairs[key] = pairs.get(key, 0) + 1
        if len(pairs) == self.size():
            return self
        keys = sorted(pairs)
        self.indices = np.array([k[0] for k in keys], dtype=self.itype)
        # count * weight in the weight type, as the reference multiplies
        self.weights = (np.array([pairs[k] for k in keys], dtype=self.ftype) *
                        np.array([k[1] for k in keys], dtype=self.ftype)).astype(self.ftype)
        return self


# ------------------------------------------------------------------------------------
# resident jobs (device state kept between calls)
# ------------------------------------------------------------------------------------
class Job:
    """A clustering job whose matrix, centers, assignments and costs stay on the GPU."""

    def __init__(self, matrix, centers, *, msr=2, prior=0., weights=None, precision="fp32", seed=1,
                 ctx: Context | None = None):
        self._ctx = ctx or default_context()
        self._M = _MatrixArg(matrix)
        if hasattr(centers, "data_ptr"):
            self._C = centers
            k = centers.shape[0]
        else:
            self._C = _centers_array(self._M, centers)
            k = self._C.shape[0]
        self.k = k
        self._w = None if weights is None else (weights if hasattr(weights, "data_ptr")
                                                else np.ascontiguousarray(weights, dtype=np.float64))
        h = ctypes.c_void_p()
        check(_lib.load().mc_job_create(self._ctx.handle, self._M.ref, _p(self._C), k, _msr(msr), float(prior),
                                        _p(self._w), _PREC[precision], int(seed), ctypes.byref(h)))
        self._h = h

    @classmethod
    def from_kmeanspp(cls, matrix, k, *, msr=2, prior=0., weights=None, precision="fp32", seed=1,
                      ctx: Context | None = None):
        """A job whose k centers are seeded on the device by D^2 sampling with U(seed, i): the
        centers minicore.cluster() passes from kmeanspp to hcluster
        (python/minicore/__init__.py:235-261).  The seed row ids are in ``center_ids``."""
        self = cls.__new__(cls)
        self._ctx = ctx or default_context()
        self._M = _MatrixArg(matrix)
        self._C = None
        self.k = int(k)
        self._w = None if weights is None else (weights if hasattr(weights, "data_ptr")
                                                else np.ascontiguousarray(weights, dtype=np.float64))
        self.center_ids = np.empty(self.k, dtype=np.uint32)
        h = ctypes.c_void_p()
        check(_lib.load().mc_job_create_kmeanspp(self._ctx.handle, self._M.ref, self.k, _msr(msr), float(prior),
                                                 _p(self._w), _PREC[precision], int(seed), _p(self.center_ids),
                                                 ctypes.byref(h)))
        self._h = h
        return self

    def assign(self):
        check(_lib.load().mc_job_assign(self._h))

    def lloyd_step(self) -> bool:
        r = ctypes.c_int()
        check(_lib.load().mc_job_lloyd_step(self._h, ctypes.byref(r)))
        return bool(r.value)

    def cost(self) -> float:
        c = ctypes.c_double()
        check(_lib.load().mc_job_cost(self._h, ctypes.byref(c)))
        return c.value

    def run(self, eps=1e-10, maxiter=100):
        ic, fc, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
        check(_lib.load().mc_job_run(self._h, float(eps), int(maxiter), ctypes.byref(ic), ctypes.byref(fc),
                                     ctypes.byref(it)))
        return ic.value, fc.value, it.value

    def read(self, centers=None, asn=None, costs=None):
        check(_lib.load().mc_job_read(self._h, _p(centers), _p(asn), _p(costs)))

    def recheck_count(self) -> int:
        c = ctypes.c_uint64()
        check(_lib.load().mc_job_recheck_count(self._h, ctypes.byref(c)))
        return c.value

    def close(self):
        if getattr(self, "_h", None) is not None:
            _lib.load().mc_job_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------------------------
# continuous-batching server
# ------------------------------------------------------------------------------------
class Server:
    """Continuous-batching clustering server over the mc_server_* C ABI: ``slots`` jobs run
    at once, each on its own stream; queued jobs are admitted first-fit against a device
    memory budget.  ``submit`` returns a ticket; ``wait`` returns the job's outputs and its
    queue / run / total latency."""

    def __init__(self, slots: int = 4, mem_budget: int = 0, device: int = 0):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.mc_server_create(int(device), int(slots), int(mem_budget), ctypes.byref(h)))
        self._h = h
        self._live = {}

    def submit(self, matrix, k=None, centers=None, *, msr=2, prior=0., weights=None, precision="fp32",
               eps=1e-10, maxiter=100, seed=1, outputs=True) -> int:
        """Queue one job: explicit ``centers`` (as for hcluster), or ``k`` centers seeded by
        k-means++ on the device with ``seed``.  ``outputs=False`` returns costs only."""
        M = _MatrixArg(matrix)
        if centers is not None:
            C = centers if hasattr(centers, "data_ptr") else _centers_array(M, centers)
            k = C.shape[0]
        elif k is None:
            raise ValueError("give k or centers")
        else:
            C = None
        k = int(k)
        if prior < 0:
            prior = 1.0 / M.d
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        out = {}
        if outputs:
            out["centers"] = np.empty((k, M.d), dtype=np.float32)
            out["asn"] = np.empty(M.n, dtype=np.uint32)
            out["costs"] = np.empty(M.n, dtype=np.float64)
            if C is None:
                out["center_ids"] = np.empty(k, dtype=np.uint32)
        desc = _lib.McJobDesc()
        desc.X = M.m
        desc.centers = _p(C)
        desc.k = k
        desc.msr = _msr(msr)
        desc.prior = float(prior)
        desc.weights = _p(w)
        desc.precision = _PREC[precision]
        desc.eps = float(eps)
        desc.maxiter = int(maxiter)
        desc.seed = _seed(seed)
        desc.centers_out = _p(out.get("centers"))
        desc.asn_out = _p(out.get("asn"))
        desc.costs_out = _p(out.get("costs"))
        desc.center_ids_out = _p(out.get("center_ids"))
        t = ctypes.c_uint64()
        check(self._lib.mc_server_submit(self._h, ctypes.byref(desc), ctypes.byref(t)))
        self._live[t.value] = (M, C, w, out)
        return t.value

    def _finish(self, ticket, r) -> dict:
        _, _, _, out = self._live.pop(ticket)
        if r.status != _lib.MC_OK:
            raise McError(r.status, r.error.decode(errors="replace"))
        res = {"initcost": r.initcost, "finalcost": r.finalcost, "numiter": r.numiter, "queue_ms": r.queue_ms,
               "run_ms": r.run_ms, "total_ms": r.total_ms, "setup_ms": r.setup_ms, "loop_ms": r.loop_ms,
               "read_ms": r.read_ms}
        res.update(out)
        return res

    def wait(self, ticket: int, timeout: float = 3600.0) -> dict:
        r = _lib.McJobResult()
        check(self._lib.mc_server_wait(self._h, int(ticket), int(timeout * 1000), ctypes.byref(r)))
        return self._finish(ticket, r)

    def poll(self, ticket: int):
        """The result dict, or None while the job is queued or running."""
        r = _lib.McJobResult()
        st = self._lib.mc_server_poll(self._h, int(ticket), ctypes.byref(r))
        if st == _lib.MC_EBUSY:
            return None
        check(st)
        return self._finish(ticket, r)

    def stats(self) -> dict:
        import json
        buf = ctypes.create_string_buffer(4096)
        check(self._lib.mc_server_stats(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def reset_stats(self):
        check(self._lib.mc_server_reset_stats(self._h))

    def close(self):
        if getattr(self, "_h", None) is not None:
            self._lib.mc_server_destroy(self._h)
            self._h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------------------------
# kernel-variant autotuner
# ------------------------------------------------------------------------------------
def autotune(enable: bool = True):
    """Turn the kernel-variant autotuner on or off (variants give bit-identical results;
    only speed differs).  Decisions persist in MC_AUTOTUNE_CACHE or the user cache dir."""
    check(_lib.load().mc_autotune_enable(1 if enable else 0))


def kernel_launches() -> int:
    """Kernels this process has launched through the library (graph replays included)."""
    return int(_lib.load().mc_kernel_launches())


LOOP_AUTO, LOOP_HOST, LOOP_FUSED, LOOP_GRAPH = -1, 0, 1, 2


def loop_mode(mode: int = LOOP_AUTO):
    """How Job.run / hcluster run the Lloyd loop: LOOP_HOST (a host round trip per
    decision), LOOP_FUSED (the stop rule on the device, one round trip per iteration),
    LOOP_GRAPH (the whole loop as one CUDA graph), LOOP_AUTO.  Results are identical."""
    check(_lib.load().mc_loop_mode(int(mode)))


def autotune_report() -> dict:
    import json
    buf = ctypes.create_string_buffer(1 << 20)
    check(_lib.load().mc_autotune_report(buf, len(buf)))
    return json.loads(buf.value.decode())


def autotune_reset():
    check(_lib.load().mc_autotune_reset())


def autotune_load(path: str):
    """Merge decisions from a cache file ("key<TAB>variant<TAB>ms,..." lines; later lines win)."""
    check(_lib.load().mc_autotune_load(os.fspath(path).encode()))


def autotune_save(path: str):
    """Write every decision of this process to a cache file."""
    check(_lib.load().mc_autotune_save(os.fspath(path).encode()))
