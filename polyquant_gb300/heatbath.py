"""Heat-bath selection over strings: an extension with no counterpart in the reference.

polyquant solves CI in spaces fixed by excitation levels (``POLYQUANT_DETSET::create_excitation``,
determinant_creation.cpp:148-206).  This module grows a *selected-string* space instead, in the spirit of
heat-bath CI (Holmes, Tubman, Umrigar, J. Chem. Theory Comput. 12, 3674 (2016)): a string enters when some
excitation that reaches it from a string already present can carry weight above a threshold.  The
determinants are the full product of the selected string lists of every species and spin
(``pq_ci_create_selected``), so every kernel of the library (sigma, Davidson, explicit H, properties) runs
on the space unchanged.

Criterion for a candidate string J of one species and spin, reached from a selected string I of that list:
    w_I * |h|  > eps,
where w_I is the largest |c| over the determinants that contain I (from the current ground state) and |h|
bounds the Hamiltonian elements the excitation can carry:
    double h1 h2 -> p1 p2 (same spin):  |(p1 h1 | p2 h2) - (p1 h2 | p2 h1)|,
    single h -> p: the largest of |F_hp(I)| (the same-spin single element of I) and |(p h | r s)| over
                   every pair r s of the other spin and of the other species (the single as half of an
                   opposite-spin or cross-species double).
Thresholds are applied in decreasing order and each starts from the previous selection, so the spaces are
nested and the variational energy cannot rise from one threshold to the next; with eps -> 0 every string
reachable by excitations joins and the energy is the one of the full product space.
"""
from __future__ import annotations

from typing import Dict, List, Sequence

import numpy as np

from .detset import POLYQUANT_DETSET

__all__ = ["heat_bath_ci", "gpu_solver", "string_excitations", "excitation_bounds"]


def _idx2(i: int, j: int) -> int:
    return i * (i + 1) // 2 + j if i >= j else j * (j + 1) // 2 + i


def _occ(m: int, n: int) -> List[int]:
    return [o for o in range(n) if (m >> o) & 1]


def string_excitations(m: int, n_orb: int):
    """Singles (h, p, J) and same-spin doubles (h1, h2, p1, p2, J) of the string m (bit o = orbital o)."""
    occ = _occ(m, n_orb)
    vir = [o for o in range(n_orb) if not (m >> o) & 1]
    singles = [(h, p, m ^ (1 << h) ^ (1 << p)) for h in occ for p in vir]
    doubles = []
    for a in range(len(occ)):
        for b in range(a + 1, len(occ)):
            for c in range(len(vir)):
                for d in range(c + 1, len(vir)):
                    h1, h2, p1, p2 = occ[a], occ[b], vir[c], vir[d]
                    doubles.append((h1, h2, p1, p2, m ^ (1 << h1) ^ (1 << h2) ^ (1 << p1) ^ (1 << p2)))
    return singles, doubles


def excitation_bounds(n_orb: Sequence[int], h1, eri: Dict, restricted: Sequence[int]):
    """Per species s and spin sp: the pair bound U[s][sp][pair] = max |(pair | rs)| over the pairs rs of the
    other spin of s and of both spins of the other species (0 when there is none), and the integral block
    E[s][sp] used for the same-spin elements (npair x npair, column-major as the library takes it)."""
    ns = len(n_orb)
    blk = lambda s, sp: sp % (1 if restricted[s] else 2)

    def block(a, sa, b, sb):
        key = (a, blk(a, sa), b, blk(b, sb))
        if key in eri:
            return np.asarray(eri[key])
        rkey = (b, blk(b, sb), a, blk(a, sa))
        if rkey in eri:
            return np.asarray(eri[rkey]).T
        raise KeyError(f"missing integral block {key}")

    U = [[None, None] for _ in range(ns)]
    E = [[None, None] for _ in range(ns)]
    for s in range(ns):
        npair = n_orb[s] * (n_orb[s] + 1) // 2
        for sp in range(2):
            E[s][sp] = block(s, sp, s, sp)
            u = np.zeros(npair)
            partners = [(s, 1 - sp)] + [(t, tsp) for t in range(ns) if t != s for tsp in range(2)]
            for t, tsp in partners:
                M = block(s, sp, t, tsp)  # rows: pairs of (s, sp)
                u = np.maximum(u, np.abs(M).max(axis=1))
            U[s][sp] = u
    return U, E


def _single_element(m: int, h: int, p: int, n: int, h1: np.ndarray, E: np.ndarray) -> float:
    """F_hp(I) = h_hp + sum_{k in occ(I)} ((hp|kk) - (hk|kp)) for the string m = I."""
    v = h1[h, p]
    hp = _idx2(h, p)
    for k in _occ(m, n):
        v += E[hp, _idx2(k, k)] - E[_idx2(h, k), _idx2(k, p)]
    return v


def gpu_solver(problem: dict, num_states: int = 1, convergence_E: float = 1e-9, num_subspace_vec: int = 8):
    """The default solver of ``heat_bath_ci``: the selected-string space on the GPU (``pq_ci_create_selected``)
    and its Davidson solve.  Returns (energies, ground-state vector, det_unfold)."""
    n_orb, na, nb = list(problem["n_orb"]), list(problem["n_alpha"]), list(problem["n_beta"])

    def solve(strings):
        ds = POLYQUANT_DETSET(n_orb, na, nb, problem["h1"], problem["eri"], restricted=problem.get("restricted"),
                              charge=problem.get("charge"), selected_strings=strings)
        try:
            k = min(num_states, ds.N_dets)
            if ds.N_dets == 1:
                return ds.diagonal().cpu().numpy()[:1], np.ones(1), ds.det_unfold()
            e, vecs, info = ds.davidson(num_states=k, num_subspace_vec=min(max(num_subspace_vec, 2 * k), ds.N_dets),
                                        convergence_E=convergence_E, return_vectors=True)
            return np.asarray(e), vecs[:, 0].cpu().numpy(), ds.det_unfold()
        finally:
            ds.close()

    return solve


def heat_bath_ci(problem: dict, eps: Sequence[float], num_states: int = 1, max_rounds: int = 20,
                 convergence_E: float = 1e-9, num_subspace_vec: int = 8, e_const: float = 0.0,
                 solver=None) -> List[dict]:
    """Selected-string CI for a sequence of decreasing thresholds ``eps``.

    ``problem``: the POLYQUANT_DETSET arguments (n_orb, n_alpha, n_beta, h1, eri, restricted, charge).
    ``solver(strings) -> (energies, ground-state vector, det_unfold)`` solves one selected space (default:
    ``gpu_solver``); the vector and the unfold table are in the space's determinant order (full product of
    the lists, species 0 alpha outermost).
    Returns one record per threshold: eps, energies (lowest ``num_states``, plus ``e_const``), the number of
    strings of every species and spin, the number of determinants, the selection rounds used and the
    selected strings (``strings[s][spin]``, in determinant order)."""
    n_orb = list(problem["n_orb"])
    na, nb = list(problem["n_alpha"]), list(problem["n_beta"])
    ns = len(n_orb)
    restricted = list(problem.get("restricted") or [1] * ns)
    h1, eri = problem["h1"], problem["eri"]
    if max(n_orb) > 64:
        raise ValueError("heat_bath_ci: selected string lists hold at most 64 orbitals per species")
    U, E = excitation_bounds(n_orb, h1, eri, restricted)
    hblk = [[np.asarray(h1[s][sp % len(h1[s])]) for sp in range(2)] for s in range(ns)]
    ne = [[na[s], nb[s]] for s in range(ns)]
    # start: the Hartree-Fock string of every list
    strings = [[[(1 << ne[s][sp]) - 1] for sp in range(2)] for s in range(ns)]
    members = [[set(strings[s][sp]) for sp in range(2)] for s in range(ns)]
    if solver is None:
        solver = gpu_solver(problem, num_states, convergence_E, num_subspace_vec)
    out = []
    for e in sorted(eps, reverse=True):
        rounds = 0
        while True:
            rounds += 1
            energies, c, unfold = solver(strings)
            if rounds > max_rounds:
                break
            added = 0
            for s in range(ns):
                for sp in range(2):
                    col = unfold[:, 2 * s + sp]
                    w = np.zeros(len(strings[s][sp]))
                    np.maximum.at(w, col, np.abs(c))
                    new = []
                    for i, m in enumerate(strings[s][sp]):
                        if w[i] == 0.0:
                            continue
                        singles, doubles = string_excitations(m, n_orb[s])
                        for (h, p, J) in singles:
                            if J in members[s][sp]:
                                continue
                            bound = max(abs(_single_element(m, h, p, n_orb[s], hblk[s][sp], E[s][sp])),
                                        U[s][sp][_idx2(h, p)])
                            if w[i] * bound > e:
                                members[s][sp].add(J)
                                new.append(J)
                        for (a, b, p1, p2, J) in doubles:
                            if J in members[s][sp]:
                                continue
                            Es = E[s][sp]
                            v = Es[_idx2(p1, a), _idx2(p2, b)] - Es[_idx2(p1, b), _idx2(p2, a)]
                            if w[i] * abs(v) > e:
                                members[s][sp].add(J)
                                new.append(J)
                    strings[s][sp] = strings[s][sp] + new
                    added += len(new)
            if added == 0:
                break
        out.append(dict(eps=float(e), energies=[float(x) + e_const for x in np.atleast_1d(energies)[:num_states]],
                        n_strings=[[len(strings[s][sp]) for sp in range(2)] for s in range(ns)],
                        n_dets=int(np.prod([len(strings[s][sp]) for s in range(ns) for sp in range(2)])),
                        rounds=rounds, strings=[[list(strings[s][sp]) for sp in range(2)] for s in range(ns)]))
    return out
