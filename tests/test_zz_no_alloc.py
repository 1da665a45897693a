"""mc_assign_sqrl2_noalloc: the dense SQRL2 assignment for callers that cannot allocate
device memory on the call path (hosts that reserve their GPU memory budget up front, or
that only pass the library buffers they own).  It must give the same assignments and costs
as mc_assign with MC_FP32, call after call, while its scratch lives in one fixed device
array.  This file is collected last so that a failure here comes after every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIB = 1 << 20


def _data(n, d, k, seed):
    rng = np.random.default_rng(seed)
    mu = rng.normal(size=(k, d)) * 3.0
    X = (mu[rng.integers(0, k, n)] + rng.normal(size=(n, d))).astype(np.float32)
    C = X[rng.choice(n, k, replace=False)].copy()
    return X, C


def _env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import minicore_gb300 as mc
    from minicore_gb300 import _lib
    return torch, mc, _lib, _lib.load()


def _reference(mc, _lib, lib, X, C):
    """The existing entry point (host buffers, exact FP32 path)."""
    n, k = X.shape[0], C.shape[0]
    M = mc._MatrixArg(X)
    asn = np.empty(n, np.uint32)
    cost = np.empty(n, np.float64)
    _lib.check(lib.mc_assign(mc.default_context().handle, M.ref, mc._p(C), k, 2, 0.0, _lib.MC_FP32, mc._p(asn),
                             mc._p(cost)))
    return asn, cost


def _noalloc(torch, mc, lib, Xd, Cd, asn, cost):
    n, d = Xd.shape
    stream = torch.cuda.current_stream().cuda_stream
    return lib.mc_assign_sqrl2_noalloc(mc._p(Xd), n, d, mc._p(Cd), Cd.shape[0], mc._p(asn), mc._p(cost),
                                       ctypes.c_void_p(stream))


def test_noalloc_matches_mc_assign_twice():
    """Two shapes, two calls each.  The first call in the process sets up the scratch
    address (it may load the module that holds the 4 MiB array: a bounded one-time cost);
    no later call lowers free device memory."""
    torch, mc, _lib, lib = _env()
    first = True
    for call, (n, d, k) in enumerate([(50_000, 96, 300), (33_333, 50, 37)]):
        X, C = _data(n, d, k, seed=call)
        ref_asn, ref_cost = _reference(mc, _lib, lib, X, C)
        Xd = torch.from_numpy(X).cuda()
        Cd = torch.from_numpy(C).cuda()
        asn = torch.empty(n, dtype=torch.int32, device="cuda")
        cost = torch.empty(n, dtype=torch.float64, device="cuda")
        for rep in range(2):
            asn.fill_(-1)
            cost.fill_(-1.0)
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            _lib.check(_noalloc(torch, mc, lib, Xd, Cd, asn, cost))
            torch.cuda.synchronize()
            drop = free_before - torch.cuda.mem_get_info()[0]
            if first:
                # module load with the scratch array, rounded to the allocation granularity
                assert drop <= 8 * MIB, f"first call lowered free memory by {drop} bytes"
                first = False
            else:
                assert drop <= 0, f"call {call}.{rep} lowered free memory by {drop} bytes"
            assert np.array_equal(asn.cpu().numpy().view(np.uint32), ref_asn)
            assert np.array_equal(cost.cpu().numpy(), ref_cost)


def test_noalloc_capacity_boundary():
    """kp * d exactly at the capacity (k = 128 -> kp = 128, d = 8192: 2^20 floats) is
    accepted and equals mc_assign bit for bit; the next padded step up (k = 129 -> kp = 256)
    and one more column are refused before anything runs."""
    torch, mc, _lib, lib = _env()
    n, d, k = 3000, 8192, 128
    X, C = _data(n, d, k, seed=7)
    ref_asn, ref_cost = _reference(mc, _lib, lib, X, C)
    Xd = torch.from_numpy(X).cuda()
    Cd = torch.from_numpy(C).cuda()
    asn = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    cost = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    _lib.check(_noalloc(torch, mc, lib, Xd, Cd, asn, cost))
    torch.cuda.synchronize()
    assert np.array_equal(asn.cpu().numpy().view(np.uint32), ref_asn)
    assert np.array_equal(cost.cpu().numpy(), ref_cost)
    C129 = torch.zeros((129, d), device="cuda")
    rc = _noalloc(torch, mc, lib, Xd, C129, asn, cost)
    assert rc == _lib.MC_EINVAL and b"scratch capacity" in lib.mc_last_error()
    Xw = torch.zeros((4, d + 1), device="cuda")
    Cw = torch.zeros((k, d + 1), device="cuda")
    rc = _noalloc(torch, mc, lib, Xw, Cw, asn[:4], cost[:4])
    assert rc == _lib.MC_EINVAL and b"scratch capacity" in lib.mc_last_error()


def test_noalloc_rejects_oversize_and_foreign_pointers():
    torch, mc, _lib, lib = _env()
    d = 4096
    k = 512  # kp * d = 2^21 floats > 2^20
    Xd = torch.zeros((4, d), device="cuda")
    Cd = torch.zeros((k, d), device="cuda")
    asn = torch.empty(4, dtype=torch.int32, device="cuda")
    cost = torch.empty(4, dtype=torch.float64, device="cuda")
    rc = lib.mc_assign_sqrl2_noalloc(mc._p(Xd), 4, d, mc._p(Cd), k, mc._p(asn), mc._p(cost), None)
    assert rc == _lib.MC_EINVAL and b"scratch capacity" in lib.mc_last_error()
    Xh = np.zeros((4, 8), np.float32)
    rc = lib.mc_assign_sqrl2_noalloc(mc._p(Xh), 4, 8, mc._p(Cd), 2, mc._p(asn), mc._p(cost), None)
    assert rc == _lib.MC_EINVAL and b"current device" in lib.mc_last_error()
    if torch.cuda.device_count() > 1:
        # rows on another GPU: refused, not read across the link
        Xo = torch.zeros((4, 8), device="cuda:1")
        rc = lib.mc_assign_sqrl2_noalloc(mc._p(Xo), 4, 8, mc._p(Cd), 2, mc._p(asn), mc._p(cost), None)
        assert rc == _lib.MC_EINVAL and b"current device" in lib.mc_last_error()
