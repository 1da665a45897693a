"""CPU checks of the drop-in boundary: the C-ABI library builds for sm_103a, loads, and
exports every entry point that include/minicore_gb300.h declares (no GPU needed)."""
import ctypes
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "minicore_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mc_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_every_declared_symbol():
    from minicore_gb300 import _lib
    lib = _lib.load()
    path = _lib.library_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (mc_[a-z0-9_]+)", out))
    declared = declared_symbols()
    assert declared, "no declarations parsed"
    missing = [s for s in declared if s not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for s in declared:
        assert hasattr(lib, s)
        assert s in _lib.SIGNATURES, f"no ctypes signature for {s}"


def test_library_targets_sm_103a():
    """The build compiles every translation unit for sm_103a only, and the library says so."""
    from minicore_gb300 import _lib
    from minicore_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert b"sm_103a" in _lib.load().mc_version()


def test_host_only_entry_points():
    from minicore_gb300 import _lib
    lib = _lib.load()
    assert b"sm_103a" in lib.mc_version()
    import numpy as np
    import oracle
    u = np.empty(16)
    assert lib.mc_uniforms(7, 3, 16, u.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.array_equal(u, oracle.uniforms(7, 16, offset=3))


def test_context_create_fails_cleanly_without_gpu():
    import torch
    if torch.cuda.is_available():
        return
    from minicore_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.mc_context_create(0, ctypes.byref(h))
    assert rc != 0
    assert lib.mc_last_error()


def test_python_api_rejects_out_of_scope_options():
    import numpy as np
    import pytest
    import minicore_gb300 as mc
    X = np.zeros((4, 3), np.float32)
    with pytest.raises(NotImplementedError):
        mc.scluster(X, [0, 1], mbsize=2)


def test_struct_layouts_match_the_header(tmp_path):
    """ctypes mirrors of mc_matrix / mc_job_desc / mc_job_result have the C layout."""
    import shutil
    import subprocess
    from minicore_gb300 import _lib
    if not shutil.which("gcc"):
        import pytest
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "layout.c"
    fields = {"mc_matrix": _lib.McMatrix, "mc_job_desc": _lib.McJobDesc, "mc_job_result": _lib.McJobResult}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "minicore_gb300.h"', "int main(void) {"]
    for cname, cls in fields.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(root, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                 text=True).stdout.splitlines())
    for cname, cls in fields.items():
        assert int(out[cname]) == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(cls, f).offset, f"{cname}.{f}"


def test_server_create_fails_cleanly_without_gpu():
    import torch
    if torch.cuda.is_available():
        return
    from minicore_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.mc_server_create(0, 2, 0, ctypes.byref(h)) != 0
    assert not h.value
    assert lib.mc_server_create(0, 0, 0, ctypes.byref(h)) == _lib.MC_EINVAL
    assert lib.mc_server_destroy(None) == 0


def test_autotune_cache_roundtrip(tmp_path):
    """Autotuner decisions load from and save to the cache file (host-only logic)."""
    import json
    from minicore_gb300 import _lib
    lib = _lib.load()
    assert lib.mc_autotune_reset() == 0
    src = tmp_path / "in.tsv"
    src.write_text("csr_sparse|msr5|kpl2|g1|nnz2^11|sm103x152\t1\t0.5,0.4,0.7\n"
                   "garbage line without tabs\n"
                   "dense_sqrl2|dense|k1024|d2^7|n2^22|sm103x152\t0\t1.0,1.2\n"
                   "bad_variant\tx\t1\n")
    assert lib.mc_autotune_load(str(src).encode()) == 0
    buf = ctypes.create_string_buffer(1 << 16)
    assert lib.mc_autotune_report(buf, len(buf)) == 0
    rep = json.loads(buf.value.decode())
    ent = rep["entries"]
    assert ent["csr_sparse|msr5|kpl2|g1|nnz2^11|sm103x152"]["variant"] == 1
    assert ent["dense_sqrl2|dense|k1024|d2^7|n2^22|sm103x152"]["ms"] == [1.0, 1.2]
    assert not any(k.startswith("bad_variant") or k.startswith("garbage") for k in ent)
    dst = tmp_path / "out.tsv"
    assert lib.mc_autotune_save(str(dst).encode()) == 0
    lines = sorted(dst.read_text().splitlines())
    assert any(l.startswith("csr_sparse|msr5|kpl2|g1|nnz2^11|sm103x152\t1\t") for l in lines)
    assert lib.mc_autotune_reset() == 0
    assert lib.mc_autotune_report(buf, len(buf)) == 0
    assert json.loads(buf.value.decode())["entries"] == {}
    assert lib.mc_autotune_load(str(tmp_path / "missing.tsv").encode()) == _lib.MC_EINVAL
