"""ctypes binding of libminicore_gb300.so (the C ABI declared in include/minicore_gb300.h)."""
from __future__ import annotations

import ctypes
import os

from . import build as _build

P = ctypes.c_void_p
U64 = ctypes.c_uint64
U32 = ctypes.c_uint32
I = ctypes.c_int
D = ctypes.c_double

MC_OK, MC_EINVAL, MC_ENOMEM, MC_ETIMEOUT, MC_ECUDA, MC_ENAN, MC_EUNSUPPORTED, MC_EBUSY = range(8)
MC_FP32, MC_TF32, MC_BF16 = 0, 1, 2
MC_DENSE_F32, MC_CSR_F32 = 0, 1


class McMatrix(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("reserved", ctypes.c_int32), ("nrows", U64), ("ncols", U64),
                ("values", P), ("indices", P), ("indptr", P), ("nnz", U64)]


class McJobDesc(ctypes.Structure):
    _fields_ = [("X", McMatrix), ("centers", P), ("k", U32), ("msr", I), ("prior", D), ("weights", P),
                ("precision", I), ("eps", D), ("maxiter", U64), ("seed", U64), ("centers_out", P),
                ("asn_out", P), ("costs_out", P), ("center_ids_out", P)]


class McJobResult(ctypes.Structure):
    _fields_ = [("status", I), ("numiter", U64), ("initcost", D), ("finalcost", D), ("queue_ms", D),
                ("run_ms", D), ("total_ms", D), ("error", ctypes.c_char * 256), ("setup_ms", D), ("loop_ms", D),
                ("read_ms", D)]


# name -> (restype, argtypes); every symbol the header declares
SIGNATURES = {
    "mc_version": (ctypes.c_char_p, []),
    "mc_last_error": (ctypes.c_char_p, []),
    "mc_kernel_launches": (U64, []),
    "mc_test_tc_stall_once": (I, []),
    "mc_diag_logf_rate": (I, [I, ctypes.POINTER(D)]),
    "mc_profile_enable": (I, [I]),
    "mc_profile_reset": (I, []),
    "mc_profile_report": (I, [ctypes.c_char_p, U64]),
    "mc_context_create": (I, [I, ctypes.POINTER(P)]),
    "mc_context_destroy": (I, [P]),
    "mc_context_set_stream": (I, [P, P]),
    "mc_context_synchronize": (I, [P]),
    "mc_uniforms": (I, [U64, U64, U64, P]),
    "mc_kmeanspp": (I, [P, P, U32, I, D, P, P, P, P, P]),
    "mc_kmeanspp_greedy": (I, [P, P, U32, I, D, P, U32, U64, P, P, P]),
    "mc_kmeanspp_ex": (I, [P, P, U32, I, D, P, U32, U64, U64, P, P, P]),
    "mc_assign": (I, [P, P, P, U32, I, D, I, P, P]),
    "mc_cmp": (I, [P, P, P, U64, I, D, I, P]),
    "mc_pcmp": (I, [P, P, I, D, P]),
    "mc_hcluster": (I, [P, P, P, U32, I, D, P, D, U64, U64, I, P, P, P, P, P, P]),
    "mc_hcluster_f32": (I, [P, P, P, U32, I, D, P, D, U64, U64, I, P, P, P, P, P, P]),
    "mc_sampler_create": (I, [P, U64, U64, U64, P, I, P, P, I, D, ctypes.POINTER(P)]),
    "mc_sampler_from_probs": (I, [P, U64, P, P, ctypes.POINTER(P)]),
    "mc_sampler_info": (I, [P, ctypes.POINTER(U64), ctypes.POINTER(I), ctypes.POINTER(I)]),
    "mc_sampler_weights": (I, [P, P]),
    "mc_sampler_destroy": (I, [P]),
    "mc_sampler_probs": (I, [P, P]),
    "mc_sampler_alias": (I, [P, P, P]),
    "mc_sampler_sample": (I, [P, U64, U64, I, P, P]),
    "mc_job_create": (I, [P, P, P, U32, I, D, P, I, U64, ctypes.POINTER(P)]),
    "mc_job_destroy": (I, [P]),
    "mc_job_assign": (I, [P]),
    "mc_job_lloyd_step": (I, [P, ctypes.POINTER(I)]),
    "mc_job_cost": (I, [P, ctypes.POINTER(D)]),
    "mc_job_run": (I, [P, D, U64, ctypes.POINTER(D), ctypes.POINTER(D), ctypes.POINTER(U64)]),
    "mc_job_read": (I, [P, P, P, P]),
    "mc_job_read_f32": (I, [P, P, P, P]),
    "mc_job_minibatch": (I, [P, U64, U64, U64, U64, I, ctypes.POINTER(D), ctypes.POINTER(D), ctypes.POINTER(U64)]),
    "mc_hcluster_minibatch": (I, [P, P, P, U32, I, D, P, U64, U64, U64, U64, I, U64, I, P, P, P, ctypes.POINTER(D),
                                  ctypes.POINTER(D), ctypes.POINTER(U64)]),
    "mc_hcluster_coreset": (I, [P, P, P, U32, I, D, P, U64, U64, U64, U64, U64, I, P, P, P, ctypes.POINTER(D),
                                ctypes.POINTER(D), ctypes.POINTER(U64)]),
    "mc_scluster": (I, [P, P, P, U32, I, D, P, D, U64, D, P, P, P, ctypes.POINTER(D), ctypes.POINTER(D),
                        ctypes.POINTER(U64)]),
    "mc_job_recheck_count": (I, [P, ctypes.POINTER(U64)]),
    "mc_assign_sqrl2_noalloc": (I, [P, U64, U64, P, U32, P, P, P]),
    "mc_autotune_enable": (I, [I]),
    "mc_loop_mode": (I, [I]),
    "mc_autotune_reset": (I, []),
    "mc_autotune_load": (I, [ctypes.c_char_p]),
    "mc_autotune_save": (I, [ctypes.c_char_p]),
    "mc_autotune_report": (I, [ctypes.c_char_p, U64]),
    "mc_job_create_kmeanspp": (I, [P, P, U32, I, D, P, I, U64, P, ctypes.POINTER(P)]),
    "mc_server_create": (I, [I, U32, U64, ctypes.POINTER(P)]),
    "mc_server_submit": (I, [P, ctypes.POINTER(McJobDesc), ctypes.POINTER(U64)]),
    "mc_server_poll": (I, [P, U64, ctypes.POINTER(McJobResult)]),
    "mc_server_wait": (I, [P, U64, U64, ctypes.POINTER(McJobResult)]),
    "mc_server_stats": (I, [P, ctypes.c_char_p, U64]),
    "mc_server_reset_stats": (I, [P]),
    "mc_server_destroy": (I, [P]),
}

_lib = None


class McError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[mc status {status}] {msg}")
        self.status = status


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library.  There is no CPU fallback: a missing or stale library is
    rebuilt, and a failed build raises."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(_build.LIB):
        raise ImportError(f"minicore_gb300 CUDA library missing: {_build.LIB}")
    lib = ctypes.CDLL(_build.LIB)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != MC_OK:
        msg = load().mc_last_error().decode(errors="replace")
        if status == MC_EINVAL:
            raise ValueError(msg)
        if status == MC_EUNSUPPORTED:
            raise NotImplementedError(msg)
        if status == MC_ENOMEM:
            raise MemoryError(msg)
        raise McError(status, msg)
