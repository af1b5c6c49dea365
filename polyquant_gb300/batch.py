"""Batches of independent CI problems solved together on one GPU.

``CIBatch`` wraps ``pq_ci_batch_*`` (include/pq_ci.h): one persistent sigma
kernel per Davidson iteration over every active problem, replayed as a CUDA
graph, with the launch shape picked by the library's autotuner.  Each problem
is what one ``POLYQUANT_EPCI::run`` (src/ci/epci.cpp:575-686) would solve; the
batch requires full CI per species (a full product space).
"""
from __future__ import annotations

import ctypes
from typing import Dict, List, Sequence

import numpy as np

from . import _lib
from ._lib import PQ_FP32, PQ_FP64, check  # noqa: F401  (PQ_FP32 re-exported for callers)
from .detset import INT_MAX, make_desc


def _torch():
    import torch

    return torch


class CIBatch:
    """``problems``: list of dicts with the ``POLYQUANT_DETSET`` arguments
    (n_orb, n_alpha, n_beta, h1, eri, excitation_level and optionally
    restricted, charge, max_collective_excitation_level)."""

    def __init__(self, problems: Sequence[Dict], stream=None):
        L = _lib.load()
        n = len(problems)
        descs = (_lib.PQDesc * n)()
        keep = []
        for i, pb in enumerate(problems):
            d, k = make_desc(pb["n_orb"], pb["n_alpha"], pb["n_beta"], pb["h1"], pb["eri"], pb["excitation_level"],
                             pb.get("restricted"), pb.get("charge"),
                             pb.get("max_collective_excitation_level", INT_MAX))
            descs[i] = d
            keep.append(k)
        b = ctypes.c_void_p()
        check(L.pq_ci_batch_create(descs, n, ctypes.c_void_p(stream or 0), ctypes.byref(b)), "pq_ci_batch_create")
        self._b = b
        del keep
        self.n = n
        self.n_dets = []
        for i in range(n):
            x = ctypes.c_int64()
            check(L.pq_ci_batch_num_dets(self._b, i, ctypes.byref(x)))
            self.n_dets.append(x.value)

    def close(self):
        if getattr(self, "_b", None):
            _lib.load().pq_ci_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tuning(self):
        w, r = ctypes.c_int32(), ctypes.c_int32()
        check(_lib.load().pq_ci_batch_tuning(self._b, ctypes.byref(w), ctypes.byref(r)))
        return {"warps_per_cta": w.value, "rows_per_unit": r.value}

    def sigma(self, Cs: List, precision: int = PQ_FP64) -> List:
        """sigma_i = H_i C_i for every problem; C_i: CUDA tensors (n_i, k) float64 with the same k."""
        torch = _torch()
        assert len(Cs) == self.n
        k = Cs[0].reshape(self.n_dets[0], -1).shape[1]
        Xs = [C.reshape(self.n_dets[i], -1).t().contiguous().to(torch.float64) for i, C in enumerate(Cs)]
        Ss = [torch.empty_like(X) for X in Xs]
        cp = (ctypes.c_void_p * self.n)(*[X.data_ptr() for X in Xs])
        sp = (ctypes.c_void_p * self.n)(*[S.data_ptr() for S in Ss])
        check(_lib.load().pq_ci_batch_sigma(self._b, cp, None, k, sp, None, precision), "pq_ci_batch_sigma")
        return [S.t() for S in Ss]

    def davidson(self, num_states: int = 1, num_subspace_vec: int = 4, iteration_max: int = 500,
                 convergence_E: float = 1e-6, precision: int = PQ_FP64, max_subspace: int = 0,
                 workspace_bytes: int = 0):
        """Energies (n, num_states) and per-problem reports."""
        p = _lib.PQDavidsonParams(num_states, num_subspace_vec, max_subspace, iteration_max, convergence_E, precision,
                                  0.0, 0)
        e = np.zeros((self.n, num_states), dtype=np.float64)
        reps = (_lib.PQDavidsonReport * self.n)()
        st = _lib.load().pq_ci_batch_davidson(self._b, ctypes.byref(p), workspace_bytes, e.ctypes.data, reps)
        check(st, "pq_ci_batch_davidson")
        info = [dict(iterations=r.iterations, converged=bool(r.converged), max_residual=r.max_residual,
                     sigma_calls_fp64=r.sigma_calls_fp64, sigma_calls_fp32=r.sigma_calls_fp32, seconds=r.seconds,
                     sigma_seconds=r.sigma_seconds)
                for r in reps]
        return e, info
