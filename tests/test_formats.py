"""On-disk formats of the coreset objects (coreset.h:79-178, 279-338), checked on the host:
IndexCoreset round trips, compaction, the byte layout, and plain (uncompressed) files."""
import gzip
import struct

import numpy as np
import pytest


def test_index_coreset_roundtrip_and_layout(tmp_path):
    import minicore_gb300 as mc
    ic = mc.IndexCoreset(np.array([5, 1, 9], np.uint32), np.array([0.5, 2.0, 1.25], np.float32))
    p = tmp_path / "ic.gz"
    ic.write(p)
    raw = gzip.open(p, "rb").read()
    assert raw[:8] == struct.pack("<Q", 3)
    assert np.array_equal(np.frombuffer(raw, np.uint32, 3, 8), [5, 1, 9])
    assert np.array_equal(np.frombuffer(raw, np.float32, 3, 20), np.float32([0.5, 2.0, 1.25]))
    back = mc.IndexCoreset().read(p)
    assert np.array_equal(back.indices, ic.indices) and np.array_equal(back.weights, ic.weights)
    plain = tmp_path / "ic.bin"
    plain.write_bytes(raw)
    back2 = mc.IndexCoreset().read(plain)
    assert np.array_equal(back2.indices, ic.indices)
    trunc = tmp_path / "short.bin"
    trunc.write_bytes(raw[:15])
    with pytest.raises(RuntimeError):
        mc.IndexCoreset().read(trunc)


def test_index_coreset_compact():
    import minicore_gb300 as mc
    ic = mc.IndexCoreset([4, 2, 4, 4, 2, 7], np.float32([1.5, 2.0, 1.5, 1.5, 3.0, 0.25]))
    ic.compact()
    # (2, 2.0) x1, (2, 3.0) x1, (4, 1.5) x3, (7, 0.25) x1, ordered by (index, weight)
    assert ic.indices.tolist() == [2, 2, 4, 7]
    assert ic.weights.tolist() == [2.0, 3.0, 4.5, 0.25]
    distinct = mc.IndexCoreset([3, 1], [1.0, 2.0])
    distinct.compact()
    assert distinct.indices.tolist() == [3, 1]  # unchanged order when nothing repeats


def test_sampler_file_layout_is_read(tmp_path):
    """A file in the reference's layout parses (the device part needs a GPU, checked elsewhere)."""
    import minicore_gb300 as mc
    n = 5
    probs = np.float32([0.1, 0.2, 0.3, 0.25, 0.15])
    w = np.float32([1, 2, 3, 4, 5])
    raw = struct.pack("<QQ", n, 99) + probs.tobytes() + struct.pack("<I", 137) + w.tobytes()
    p = tmp_path / "cs.bin"
    p.write_bytes(raw)
    assert mc._read_maybe_gz(p) == raw
    gz = tmp_path / "cs.gz"
    with gzip.open(gz, "wb") as f:
        f.write(raw)
    assert mc._read_maybe_gz(gz) == raw
