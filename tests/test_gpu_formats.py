"""CoresetSampler write/read on the GPU: a sampler restored from its file has the same
probabilities, alias table and draws as the one that wrote it."""
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


@pytest.mark.parametrize("weighted", [False, True])
def test_sampler_roundtrip(mc, tmp_path, weighted):
    rng = np.random.default_rng(3)
    n, k = 5000, 12
    costs = rng.gamma(2.0, 1.0, n)
    asn = rng.integers(0, k, n).astype(np.uint32)
    w = rng.uniform(0.5, 2.0, n).astype(np.float32) if weighted else None
    cs = mc.CoresetSampler()
    cs.make_sampler(k, costs, asn, weights=w, seed=77, sens=mc.LBK)
    p = tmp_path / "cs.gz"
    cs.write(p)
    back = mc.CoresetSampler().read(p)
    assert back.np_ == n and back.seed_ == 77
    assert np.array_equal(back.get_probs(), cs.get_probs())
    pt0, at0 = cs.alias_table()
    pt1, at1 = back.alias_table()
    assert np.array_equal(pt0, pt1) and np.array_equal(at0, at1)
    for unique in (False, True):
        w0, i0 = cs.sample(700, seed=5, unique=unique)
        w1, i1 = back.sample(700, seed=5, unique=unique)
        assert np.array_equal(i0, i1) and np.array_equal(w0, w1)


def test_fl_sampler_is_not_serialized(mc, tmp_path):
    rng = np.random.default_rng(4)
    cs = mc.CoresetSampler()
    cs.make_sampler(5, rng.gamma(2.0, 1.0, 500), rng.integers(0, 5, 500).astype(np.uint32), sens=mc.FL)
    with pytest.raises(RuntimeError):
        cs.write(tmp_path / "fl.gz")
