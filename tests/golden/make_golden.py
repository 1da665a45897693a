"""Regenerate tests/golden/msr_fixtures.npz from the reference's own test sources.

Reads (as text) the vectors that minicore's distance tests use:
  * src/tests/testmsr.cpp:11-19      cv1 = {10,0,4,6,0,13} and cv4 = e_3, both resized to d=12
  * src/tests/testmsr.cpp (large)    the `lhs` / `rhs` count vectors (d=26183) of the
    MKL / REVERSE_MKL positivity check; src/tests/testmsrcsr.cpp holds the same pair and is
    asserted to agree across sparse representations within 1e-5.
Usage:  python tests/golden/make_golden.py /path/to/minicore   (or MINICORE_REFERENCE=/path/to/minicore)
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _vec(src: str, pattern: str):
    m = re.search(pattern, src)
    if not m:
        raise SystemExit(f"pattern not found: {pattern}")
    return np.array([float(x) for x in m.group(1).split(",") if x.strip()], dtype=np.float64)


def main(ref_root: str) -> None:
    tdir = os.path.join(ref_root, "src", "tests")
    s = open(os.path.join(tdir, "testmsr.cpp")).read()
    s2 = open(os.path.join(tdir, "testmsrcsr.cpp")).read()
    cv1 = _vec(s, r"CompressedVector<FT>\s+cv1\{\{([^}]*)\}\}")
    cv4 = _vec(s, r"CompressedVector<FT>\s+cv4\s*=\s*\{([^}]*)\}")
    d = 12  # cv1.resize(12); cv4.resize(12) (testmsr.cpp:19-20)
    cv1 = np.pad(cv1, (0, d - cv1.size))
    cv4 = np.pad(cv4, (0, d - cv4.size))
    lhs = _vec(s, r"blz::SV<float>\s+lhs\s*\{([^}]*)\}")
    rhs = _vec(s, r"blz::SV<float>\s+rhs\s*\{([^}]*)\}")
    lhs2 = _vec(s2, r"blz::SV<float>\s+lhs\s*\{([^}]*)\}")
    rhs2 = _vec(s2, r"blz::SV<float>\s+rhs\s*\{([^}]*)\}")
    assert np.array_equal(lhs, lhs2) and np.array_equal(rhs, rhs2)
    li, ri = np.nonzero(lhs)[0], np.nonzero(rhs)[0]
    np.savez_compressed(
        os.path.join(HERE, "msr_fixtures.npz"),
        cv1=cv1.astype(np.float32), cv4=cv4.astype(np.float32),
        big_dim=np.int64(lhs.size),
        lhs_idx=li.astype(np.uint32), lhs_val=lhs[li].astype(np.float32),
        rhs_idx=ri.astype(np.uint32), rhs_val=rhs[ri].astype(np.float32),
    )
    print("wrote", os.path.join(HERE, "msr_fixtures.npz"), "d(big)=", lhs.size, "nnz:", li.size, ri.size)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MINICORE_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <path to the minicore source tree> (or set MINICORE_REFERENCE)")
    main(ref)
