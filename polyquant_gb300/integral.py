"""Host-side mirror of polyquant's integral transforms on the GB300 library.

``transform_mo_2_body_integrals`` keeps the reference's argument list
(src/integral/integral.hpp:201-204, integral.cpp:207-477): species indices,
MO coefficients (n_ao x n_mo_total), particle counts, frozen-core and
deleted-virtual counts per species; it returns the (npair_a x npair_b) matrix
at [idx2(i,j), idx2(k,l)] as a torch CUDA tensor (column-major storage exposed
as a transposed view, so element [r, c] is (r | c)).  The AO integrals are an
input here (the reference computes them inside the first quarter transform
with libint).
"""
from __future__ import annotations

import ctypes
from typing import Dict, List, Sequence, Tuple

from . import _lib
from ._lib import PQ_AO_PACKED8, PQ_AO_PAIRS, PQ_XFORM_BF16X3, PQ_XFORM_FP64, PQ_XFORM_TF32X3, check  # noqa: F401


def _torch():
    import torch

    return torch


def ao2mo(eri_ao, C_a, C_b=None, layout: int = PQ_AO_PACKED8, mode: int = PQ_XFORM_FP64, stream=None):
    """(ij|kl) for all i>=j, k>=l from device AO integrals and MO coefficients.

    eri_ao: torch float64 CUDA tensor, 8-fold packed (layout PQ_AO_PACKED8) or
    an (npair_a x npair_b) pair matrix in column-major storage (PQ_AO_PAIRS,
    pass the transpose of a row-major tensor).  C_a, C_b: (n_ao x n_mo).
    Returns an (npair_mo_a x npair_mo_b) tensor.
    """
    torch = _torch()
    same = C_b is None
    C_b = C_a if same else C_b
    na, nma = C_a.shape
    nb, nmb = C_b.shape
    # column-major (n_ao x n_mo) storage == row-major (n_mo x n_ao)
    Ca = C_a.t().contiguous().to(torch.float64)
    Cb = Ca if same else C_b.t().contiguous().to(torch.float64)
    npa, npb = nma * (nma + 1) // 2, nmb * (nmb + 1) // 2
    out = torch.empty((npb, npa), dtype=torch.float64, device=Ca.device)
    st = ctypes.c_void_p(stream or torch.cuda.current_stream().cuda_stream)
    check(_lib.load().pq_ao2mo(ctypes.c_void_p(eri_ao.data_ptr()), layout, na, nb, ctypes.c_void_p(Ca.data_ptr()), na,
                               nma, ctypes.c_void_p(Cb.data_ptr()), nb, nmb, mode, ctypes.c_void_p(out.data_ptr()), st),
          "pq_ao2mo")
    return out.t()


def transform_mo_2_body_integrals(a: int, b: int, mo_coeffs_a, mo_coeffs_b, num_part_alpha: int, num_part_beta: int,
                                  frozen_core, deleted_virtual, eri_ao, layout: int = PQ_AO_PACKED8,
                                  mode: int = PQ_XFORM_FP64):
    """Reference signature (integral.hpp:201-204): active MO range
    [frozen_core, n_mo - deleted_virtual) of each species, as integral.cpp:215-218."""
    nmo_a = mo_coeffs_a.shape[1] - frozen_core[a] - deleted_virtual[a]
    nmo_b = mo_coeffs_b.shape[1] - frozen_core[b] - deleted_virtual[b]
    Ca = mo_coeffs_a[:, frozen_core[a]:frozen_core[a] + nmo_a]
    Cb = mo_coeffs_b[:, frozen_core[b]:frozen_core[b] + nmo_b]
    same = (mo_coeffs_a is mo_coeffs_b) and frozen_core[a] == frozen_core[b] and deleted_virtual[a] == deleted_virtual[b]
    return ao2mo(eri_ao, Ca, None if same else Cb, layout=layout, mode=mode)


def calculate_mo_1_body_integrals(F_ao, mo_coeffs, frozen_core: int = 0, deleted_virtual: int = 0, stream=None):
    """h_MO = C^T F C over the active MOs (integral.cpp:166-205)."""
    torch = _torch()
    nmo = mo_coeffs.shape[1] - frozen_core - deleted_virtual
    C = mo_coeffs[:, frozen_core:frozen_core + nmo].t().contiguous().to(torch.float64)
    F = F_ao.t().contiguous().to(torch.float64)  # column-major F (symmetric in practice)
    n = F_ao.shape[0]
    out = torch.empty((nmo, nmo), dtype=torch.float64, device=C.device)
    st = ctypes.c_void_p(stream or torch.cuda.current_stream().cuda_stream)
    check(_lib.load().pq_mo1(ctypes.c_void_p(F.data_ptr()), n, ctypes.c_void_p(C.data_ptr()), n, nmo,
                             ctypes.c_void_p(out.data_ptr()), st), "pq_mo1")
    return out.t()


def calculate_mo_2_body_integrals(mo_coeffs: Sequence[Sequence], frozen_core: Sequence[int],
                                  deleted_virtual: Sequence[int], eri_ao: Dict[Tuple[int, int], object],
                                  num_parts: Sequence[Tuple[int, int]] = None, layout: int = PQ_AO_PACKED8,
                                  mode: int = PQ_XFORM_FP64) -> List[List[List[List[object]]]]:
    """mo_two_body_ints[a][sa][b][sb] for every species pair b >= a and every spin block of each
    (calculate_mo_2_body_integrals, integral.cpp:479-516; entries with b < a stay None, as the reference leaves
    them empty).  mo_coeffs[s][spin]: (n_ao x n_mo) device tensors, one per spin block; eri_ao[(a, b)]: the AO
    integrals of the species pair in ``layout``; num_parts[s] = (alpha, beta) particle counts, passed through
    as the reference does."""
    ns = len(mo_coeffs)
    parts = num_parts if num_parts is not None else [(0, 0)] * ns
    out: List[List[List[List[object]]]] = []
    for a in range(ns):
        per_a = []
        for sa in range(len(mo_coeffs[a])):
            per_b = []
            for b in range(ns):
                blocks = [None] * len(mo_coeffs[b])
                if b >= a:
                    for sb in range(len(mo_coeffs[b])):
                        blocks[sb] = transform_mo_2_body_integrals(
                            a, b, mo_coeffs[a][sa], mo_coeffs[b][sb], parts[a][sa], parts[b][sb], frozen_core,
                            deleted_virtual, eri_ao[(a, b)], layout=layout, mode=mode)
                per_b.append(blocks)
            per_a.append(per_b)
        out.append(per_a)
    return out
