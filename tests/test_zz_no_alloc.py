"""mc_assign_sqrl2_noalloc: the dense SQRL2 assignment for callers that cannot allocate
device memory on the call path (hosts that reserve their GPU memory budget up front, or
that only pass the library buffers they own).  It must give the same assignments and costs
as mc_assign with MC_FP32, call after call, while its scratch lives in one fixed device
array.  This file is collected last so that a failure here comes after every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n, d, k, seed):
    rng = np.random.default_rng(seed)
    mu = rng.normal(size=(k, d)) * 3.0
    X = (mu[rng.integers(0, k, n)] + rng.normal(size=(n, d))).astype(np.float32)
    C = X[rng.choice(n, k, replace=False)].copy()
    return X, C


def test_noalloc_matches_mc_assign_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import minicore_gb300 as mc
    from minicore_gb300 import _lib
    lib = _lib.load()
    ctx = mc.default_context()
    stream = torch.cuda.current_stream().cuda_stream
    for call, (n, d, k) in enumerate([(50_000, 96, 300), (33_333, 50, 37)]):
        X, C = _data(n, d, k, seed=call)
        # reference: the existing entry point (host buffers, FP32 path)
        M = mc._MatrixArg(X)
        ref_asn = np.empty(n, np.uint32)
        ref_cost = np.empty(n, np.float64)
        _lib.check(lib.mc_assign(ctx.handle, M.ref, mc._p(C), k, 2, 0.0, _lib.MC_FP32, mc._p(ref_asn),
                                 mc._p(ref_cost)))
        Xd = torch.from_numpy(X).cuda()
        Cd = torch.from_numpy(C).cuda()
        asn = torch.empty(n, dtype=torch.int32, device="cuda")
        cost = torch.empty(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free_before = None
        for rep in range(2):
            asn.fill_(-1)
            cost.fill_(-1.0)
            _lib.check(lib.mc_assign_sqrl2_noalloc(mc._p(Xd), n, d, mc._p(Cd), k, mc._p(asn), mc._p(cost),
                                                   ctypes.c_void_p(stream)))
            torch.cuda.synchronize()
            if rep == 0:
                free_before = torch.cuda.mem_get_info()[0]
            else:
                assert torch.cuda.mem_get_info()[0] == free_before  # the call allocated nothing
            assert np.array_equal(asn.cpu().numpy().view(np.uint32), ref_asn)
            assert np.array_equal(cost.cpu().numpy(), ref_cost)


def test_noalloc_rejects_oversize_and_host_pointers():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import minicore_gb300 as mc
    from minicore_gb300 import _lib
    lib = _lib.load()
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
    assert rc == _lib.MC_EINVAL
