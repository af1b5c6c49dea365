"""Seeded synthetic inputs for the CI sigma and AO->MO workloads.

These stand in for the reference's libint-generated integrals on the
benchmark workloads (no integral engine is part of this path):

* ``fci_integrals``: one species, n spatial orbitals.  h_pq symmetric with
  h_pp = -(20 - p) and off-diagonals N(0, 0.1) exp(-|p-q|/4);
  (pq|rs) = sum_L B_Lpq B_Lrs with B_Lpq = B_Lqp ~ N(0, 0.15) exp(-|p-q|/3), so
  the tensor is 8-fold symmetric and positive semidefinite.
* ``ep_integrals``: electron + positron blocks built the same way with
  separate seeds; the e-p block is (pq|rs)_ep = sum_L B^e_Lpq B^p_Lrs.
* ``ao_eri_packed8``: (mu nu|la si) = sum_L B_L,mu nu B_L,la si with
  B ~ N(0, 1) exp(-|mu - nu|/16), returned 8-fold packed.
* ``mo_coefficients``: Q factor of a seeded Gaussian matrix.

All integral matrices use the reference layout: pair index
idx2(i, j) = max(i,j)(max(i,j)+1)/2 + min(i,j) (integral.hpp:14-20) and the ERI
block is an (npair_a x npair_b) matrix at [idx2(i,j), idx2(k,l)].
"""
from __future__ import annotations

import numpy as np


def pair_index(n: int):
    """(i, j) arrays of the idx2 ordering: pair k <-> (i_k >= j_k)."""
    i, j = np.tril_indices(n)
    return i, j


def _pair_matrix(B: np.ndarray) -> np.ndarray:
    """B[L, p, q] (symmetric in p, q) -> Bp[L, pair]."""
    n = B.shape[1]
    i, j = pair_index(n)
    return B[:, i, j]


def _sym_noise(rng, L, n, sigma, decay):
    d = np.abs(np.arange(n)[:, None] - np.arange(n)[None, :])
    B = rng.standard_normal((L, n, n)) * sigma * np.exp(-d / decay)
    return 0.5 * (B + B.transpose(0, 2, 1))


def one_body(rng, n: int) -> np.ndarray:
    d = np.abs(np.arange(n)[:, None] - np.arange(n)[None, :])
    h = rng.standard_normal((n, n)) * 0.1 * np.exp(-d / 4.0)
    h = 0.5 * (h + h.T)
    h[np.arange(n), np.arange(n)] = -(20.0 - np.arange(n))
    return h


def fci_integrals(n: int, seed: int = 0, L: int = 48):
    """(h, eri_pairs) for one restricted species with n orbitals."""
    rng = np.random.default_rng(seed)
    h = one_body(rng, n)
    Bp = _pair_matrix(_sym_noise(rng, L, n, 0.15, 3.0))
    eri = Bp.T @ Bp
    return h, np.ascontiguousarray(eri)


def ep_integrals(n_e: int, n_p: int, seed: int = 0, L: int = 48):
    """Electron, positron and e-p blocks: (h_e, h_p, eri_ee, eri_pp, eri_ep)."""
    rng_e = np.random.default_rng(seed)
    rng_p = np.random.default_rng(seed + 7919)
    h_e = one_body(rng_e, n_e)
    h_p = one_body(rng_p, n_p)
    Be = _pair_matrix(_sym_noise(rng_e, L, n_e, 0.15, 3.0))
    Bq = _pair_matrix(_sym_noise(rng_p, L, n_p, 0.15, 3.0))
    return h_e, h_p, Be.T @ Be, Bq.T @ Bq, Be.T @ Bq


def ao_eri_pairs(n: int, seed: int = 0, L: int = 1024, xp=np):
    """Factor Bp[L, npair] of the AO ERIs; (mu nu|la si) = (Bp^T Bp)[mu nu, la si]."""
    rng = np.random.default_rng(seed)
    d = np.abs(np.arange(n)[:, None] - np.arange(n)[None, :])
    i, j = pair_index(n)
    Bp = np.empty((L, len(i)), dtype=np.float64)
    decay = np.exp(-d / 16.0)[i, j]
    for l0 in range(0, L, 64):
        l1 = min(L, l0 + 64)
        B = rng.standard_normal((l1 - l0, n, n))
        B = 0.5 * (B + B.transpose(0, 2, 1))
        Bp[l0:l1] = B[:, i, j] * decay
    return Bp


def mo_coefficients(n_ao: int, n_mo: int = None, seed: int = 1) -> np.ndarray:
    n_mo = n_ao if n_mo is None else n_mo
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((n_ao, n_ao)))
    return np.ascontiguousarray(q[:, :n_mo])


def packed8_from_pairs(M: np.ndarray) -> np.ndarray:
    """Lower triangle of the symmetric pair matrix, packed by idx2(pair, pair)."""
    a, b = np.tril_indices(M.shape[0])
    return np.ascontiguousarray(M[a, b])


def ao_eri_packed8(n: int, seed: int = 0, L: int = 1024) -> np.ndarray:
    """8-fold packed AO ERIs (host numpy; intended for small n)."""
    Bp = ao_eri_pairs(n, seed, L)
    return packed8_from_pairs(Bp.T @ Bp)


def batch_specs(n_problems: int = 256, seed: int = 0, n_pos_orb: int = 6):
    """Shapes of the batched uneven-CI workload: n_orb ~ U{8..14}, n_alpha, n_beta ~ U{2..n_orb//2},
    0-2 positrons (1 = one alpha positron, 2 = one alpha + one beta) in n_pos_orb orbitals; each
    problem's integrals use seed * 100003 + index."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_problems):
        n = int(rng.integers(8, 15))
        a = int(rng.integers(2, n // 2 + 1))
        b = int(rng.integers(2, n // 2 + 1))
        npos = int(rng.integers(0, 3))
        specs.append(dict(n_orb=n, n_alpha=a, n_beta=b, n_pos=npos, n_pos_orb=n_pos_orb, seed=seed * 100003 + i))
    return specs


def _comb(n, k):
    from math import comb

    return comb(n, k)


def batch_spec_dets(s) -> int:
    p = {0: 1, 1: s["n_pos_orb"], 2: s["n_pos_orb"] ** 2}[s["n_pos"]]
    return _comb(s["n_orb"], s["n_alpha"]) * _comb(s["n_orb"], s["n_beta"]) * p


def batch_problem(s) -> dict:
    """Full-CI problem of one spec as keyword arguments of POLYQUANT_DETSET / CIBatch."""
    n, a, b = s["n_orb"], s["n_alpha"], s["n_beta"]
    ex_e = [min(a, n - a), min(b, n - b), min(a, n - a) + min(b, n - b)]
    if s["n_pos"] == 0:
        h, eri = fci_integrals(n, s["seed"])
        return dict(n_orb=[n], n_alpha=[a], n_beta=[b], h1=[[h]], eri={(0, 0, 0, 0): eri}, excitation_level=[ex_e],
                    restricted=[1], charge=[-1.0])
    m = s["n_pos_orb"]
    pa, pb = (1, 0) if s["n_pos"] == 1 else (1, 1)
    h_e, h_p, ee, pp, ep = ep_integrals(n, m, s["seed"])
    ex_p = [min(pa, m - pa), min(pb, m - pb), min(pa, m - pa) + min(pb, m - pb)]
    return dict(n_orb=[n, m], n_alpha=[a, pa], n_beta=[b, pb], h1=[[h_e], [h_p]],
                eri={(0, 0, 0, 0): ee, (1, 0, 1, 0): pp, (0, 0, 1, 0): ep}, excitation_level=[ex_e, ex_p],
                restricted=[1, 1], charge=[-1.0, 1.0])
