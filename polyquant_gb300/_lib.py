"""ctypes binding of libpq_gb300.so (the C ABI in include/pq_ci.h, include/pq_ints.h).

The library is the only compute path: loading fails loudly when it has not been
built, and every entry point that returns a non-zero pq_status raises.
"""
from __future__ import annotations

import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libpq_gb300.so")

PQ_OK, PQ_ERR_ARG, PQ_ERR_CUDA, PQ_ERR_OOM, PQ_NOT_CONVERGED, PQ_TIMEOUT, PQ_ERR_STATE = range(7)
PQ_FP64, PQ_FP32 = 0, 1
PQ_AO_PACKED8, PQ_AO_PAIRS = 0, 1
PQ_XFORM_FP64, PQ_XFORM_BF16X3, PQ_XFORM_TF32X3 = 0, 1, 2

EXPORTS = [
    "pq_last_error", "pq_version", "pq_ci_create", "pq_ci_create_selected", "pq_ci_destroy", "pq_ci_num_dets", "pq_ci_strings",
    "pq_ci_det_unfold", "pq_ci_diag", "pq_ci_sigma", "pq_ci_sigma_host", "pq_ci_sigma_noalloc",
    "pq_ci_sigma_interleaved", "pq_ci_element", "pq_ci_elements", "pq_debug_scratch_bytes",
    "pq_ci_davidson", "pq_ci_ham_build", "pq_ci_ham_release", "pq_ci_ham_csr", "pq_ci_s2", "pq_ci_rdm1",
    "pq_ci_batch_create", "pq_ci_batch_destroy", "pq_ci_batch_num_dets", "pq_ci_batch_sigma",
    "pq_ci_batch_tuning", "pq_ci_batch_davidson", "pq_ao2mo", "pq_mo1", "pq_debug_set_wait_budget",
    "pq_ao2mo_release_workspace",
]


class PQError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"pq_status {status}: {msg}")
        self.status = status


class PQDesc(ctypes.Structure):
    """pq_ci_desc (include/pq_ci.h)."""

    _fields_ = [
        ("n_species", ctypes.c_int32),
        ("n_orb", ctypes.c_int32 * 2),
        ("n_alpha", ctypes.c_int32 * 2),
        ("n_beta", ctypes.c_int32 * 2),
        ("restricted", ctypes.c_int32 * 2),
        ("charge", ctypes.c_double * 2),
        ("ex_level", (ctypes.c_int32 * 3) * 2),
        ("max_collective", ctypes.c_int32),
        ("h1", (ctypes.c_void_p * 2) * 2),
        ("eri", ((((ctypes.c_void_p * 2) * 2) * 2) * 2)),
    ]


class PQDavidsonParams(ctypes.Structure):
    _fields_ = [
        ("num_states", ctypes.c_int32),
        ("num_subspace_vec", ctypes.c_int32),
        ("max_subspace", ctypes.c_int32),
        ("iteration_max", ctypes.c_int32),
        ("convergence_E", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("energy_shift", ctypes.c_double),
        ("verbose", ctypes.c_int32),
    ]


class PQDavidsonReport(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int32),
        ("sigma_calls_fp64", ctypes.c_int32),
        ("sigma_calls_fp32", ctypes.c_int32),
        ("converged", ctypes.c_int32),
        ("max_residual", ctypes.c_double),
        ("seconds", ctypes.c_double),
        ("sigma_seconds", ctypes.c_double),
    ]


_lib = None


def load(path: str = LIB_PATH):
    """Load the library (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    P, I32, I64, D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    L.pq_last_error.restype = ctypes.c_char_p
    L.pq_version.restype = ctypes.c_char_p
    L.pq_ci_create.restype = I32
    L.pq_ci_create.argtypes = [ctypes.POINTER(PQDesc), P, ctypes.POINTER(P)]
    L.pq_ci_create_selected.restype = I32
    L.pq_ci_create_selected.argtypes = [ctypes.POINTER(PQDesc), P, P, P, ctypes.POINTER(P)]
    L.pq_ci_destroy.restype = I32
    L.pq_ci_destroy.argtypes = [P]
    L.pq_ci_num_dets.restype = I32
    L.pq_ci_num_dets.argtypes = [P, ctypes.POINTER(I64)]
    L.pq_ci_strings.restype = I32
    L.pq_ci_strings.argtypes = [P, I32, I32, P, ctypes.POINTER(I64), ctypes.POINTER(I32)]
    L.pq_ci_det_unfold.restype = I32
    L.pq_ci_det_unfold.argtypes = [P, P]
    L.pq_ci_diag.restype = I32
    L.pq_ci_diag.argtypes = [P, P]
    for f in (L.pq_ci_sigma, L.pq_ci_sigma_host, L.pq_ci_sigma_noalloc):
        f.restype = I32
        f.argtypes = [P, P, I64, I32, P, I64, I32]
    L.pq_ci_element.restype = I32
    L.pq_ci_element.argtypes = [P, I64, I64, ctypes.POINTER(D)]
    L.pq_ci_elements.restype = I32
    L.pq_ci_elements.argtypes = [P, I64, P, P, P]
    L.pq_debug_scratch_bytes.restype = I32
    L.pq_debug_scratch_bytes.argtypes = [P, ctypes.POINTER(I64)]
    L.pq_ci_sigma_interleaved.restype = I32
    L.pq_ci_sigma_interleaved.argtypes = [P, P, P, I32, I32, D]
    L.pq_ci_davidson.restype = I32
    L.pq_ci_davidson.argtypes = [P, ctypes.POINTER(PQDavidsonParams), P, P, ctypes.POINTER(PQDavidsonReport)]
    L.pq_ci_ham_build.restype = I32
    L.pq_ci_ham_build.argtypes = [P, D, I32, ctypes.POINTER(I64)]
    L.pq_ci_ham_release.restype = I32
    L.pq_ci_ham_release.argtypes = [P]
    L.pq_ci_ham_csr.restype = I32
    L.pq_ci_ham_csr.argtypes = [P, I32, ctypes.POINTER(I64), P, P, P]
    L.pq_ci_s2.restype = I32
    L.pq_ci_s2.argtypes = [P, P, I64, I32, P]
    L.pq_ci_rdm1.restype = I32
    L.pq_ci_rdm1.argtypes = [P, P, I32, I32, P]
    L.pq_ci_batch_create.restype = I32
    L.pq_ci_batch_create.argtypes = [ctypes.POINTER(PQDesc), I32, P, ctypes.POINTER(P)]
    L.pq_ci_batch_destroy.restype = I32
    L.pq_ci_batch_destroy.argtypes = [P]
    L.pq_ci_batch_num_dets.restype = I32
    L.pq_ci_batch_num_dets.argtypes = [P, I32, ctypes.POINTER(I64)]
    L.pq_ci_batch_sigma.restype = I32
    L.pq_ci_batch_sigma.argtypes = [P, P, P, I32, P, P, I32]
    L.pq_ci_batch_tuning.restype = I32
    L.pq_ci_batch_tuning.argtypes = [P, ctypes.POINTER(I32), ctypes.POINTER(I32)]
    L.pq_ci_batch_davidson.restype = I32
    L.pq_ci_batch_davidson.argtypes = [P, ctypes.POINTER(PQDavidsonParams), ctypes.c_size_t, P,
                                       ctypes.POINTER(PQDavidsonReport)]
    L.pq_ao2mo.restype = I32
    L.pq_ao2mo.argtypes = [P, I32, I64, I64, P, I64, I64, P, I64, I64, I32, P, P]
    L.pq_ao2mo_release_workspace.restype = I32
    L.pq_ao2mo_release_workspace.argtypes = []
    L.pq_debug_set_wait_budget.restype = I32
    L.pq_debug_set_wait_budget.argtypes = [ctypes.c_longlong]
    L.pq_mo1.restype = I32
    L.pq_mo1.argtypes = [P, I64, P, I64, I64, P, P]
    _lib = L
    return L


def check(status: int, what: str = "") -> int:
    if status != PQ_OK and status != PQ_NOT_CONVERGED:
        msg = load().pq_last_error().decode()
        raise PQError(status, f"{what}: {msg}" if what else msg)
    return status


def last_error() -> str:
    return load().pq_last_error().decode()
