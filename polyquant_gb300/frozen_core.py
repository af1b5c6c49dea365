"""Frozen-core operator and energy, the setup step in front of an active-space CI.

Restates, on the host (the reference also forms them once, on the CPU, before
the CI):

* the frozen-core density of each species and spin block, C[:, :n_fc] C[:, :n_fc]^T
  with occupation 1 per orbital (fc_dm, src/ci/epci.cpp:52-95);
* POLYQUANT_INTEGRAL::calculate_frozen_core_ints / compute_frozen_core_ints
  (src/integral/integral.cpp:64-95, 569-699): for species a and spin block s
      F_fc[a][s] = T/m - q_a V + sum over species b with frozen orbitals of
                   q J_ab(D_b) - K_aa(D_a,s)   (exchange within a species only),
  with D_b the total frozen density of b, the Coulomb term carrying
  charge[a] * charge[b] between species and 1 within one, and the exchange
  taken with the spin block's own density;
* the frozen-core energy per species (epci.cpp:110-128):
      restricted    sum D_a,0 * (H_core + F_fc[a][0])
      unrestricted  0.5 sum [(D_0 + D_1) * H_core + D_0 * F_fc[0] + D_1 * F_fc[1]].

The active-space one-body integrals are then C_act^T F_fc C_act
(``integral.calculate_mo_1_body_integrals`` on the device), and the CI
energies are shifted by E_nuc + sum of the frozen-core energies
(epci.cpp:595-614).

Two details of the reference's compute_frozen_core_ints are reproduced by
default, so that the results equal the reference's on the same inputs: the
charge product is converted to an integer, and the cross-species Coulomb
term of a partner species with two spin blocks (unrestricted) is added once
per block, each time with the partner's total frozen density -- the same
per-block count the reference's SCF Fock build makes.  With
``single_count_cross=True`` the partner's density enters once with the exact
charge product (the physical operator, for which the frozen-block identity
of the tests holds).  Restricted or single-block partners with charges of +-1
are the same either way.
"""
from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy as np


def frozen_core_density(mo_coeffs: np.ndarray, n_frozen: int) -> np.ndarray:
    """C[:, :n_frozen] C[:, :n_frozen]^T (occupation 1 per frozen orbital)."""
    c = np.asarray(mo_coeffs, dtype=np.float64)[:, :n_frozen]
    return c @ c.T


def _total(dm: Sequence[np.ndarray], restricted: bool) -> np.ndarray:
    return 2.0 * dm[0] if restricted or len(dm) == 1 else dm[0] + dm[1]


def _cross(eri_ao: Dict[Tuple[int, int], np.ndarray], a: int, b: int, D: np.ndarray) -> np.ndarray:
    """sum_kl (ij|kl)_ab D_kl for species a's pair ij and species b's pair kl."""
    if (a, b) in eri_ao:
        return np.einsum("ijkl,kl->ij", eri_ao[(a, b)], D, optimize=True)
    return np.einsum("klij,kl->ij", eri_ao[(b, a)], D, optimize=True)


def calculate_frozen_core_ints(hcore: Sequence[np.ndarray], fc_dm: Sequence[Sequence[np.ndarray]],
                               frozen_core: Sequence[int], eri_ao: Dict[Tuple[int, int], np.ndarray],
                               charge: Sequence[float], restricted: Sequence[bool],
                               single_count_cross: bool = False) -> List[List[np.ndarray]]:
    """F_fc[a][spin] in the AO basis.

    hcore[a]      T / mass - charge * V of species a (AO, n_a x n_a)
    fc_dm[a]      frozen-core densities per spin block (one block for a restricted species)
    eri_ao[(a,b)] full AO Coulomb tensors (n_a, n_a, n_b, n_b) for each species pair, a <= b
    """
    ns = len(hcore)
    F = []
    for a in range(ns):
        Fa = []
        for s in range(len(fc_dm[a])):
            f = np.array(hcore[a], dtype=np.float64, copy=True)
            for b in range(ns):
                if frozen_core[b] == 0:
                    continue
                Dt = _total(fc_dm[b], restricted[b])
                if b == a:
                    f += _cross(eri_ao, a, a, Dt)
                    Ds = fc_dm[a][0] if restricted[a] else fc_dm[a][s]
                    f -= np.einsum("ikjl,kl->ij", eri_ao[(a, a)], Ds, optimize=True)
                elif single_count_cross:
                    f += charge[a] * charge[b] * _cross(eri_ao, a, b, Dt)
                else:
                    blocks = 1 if restricted[b] else len(fc_dm[b])
                    f += blocks * int(charge[a] * charge[b]) * _cross(eri_ao, a, b, Dt)
            Fa.append(f)
        F.append(Fa)
    return F


def frozen_core_energy(hcore: Sequence[np.ndarray], fc_dm: Sequence[Sequence[np.ndarray]],
                       F_fc: Sequence[Sequence[np.ndarray]], frozen_core: Sequence[int],
                       restricted: Sequence[bool]) -> List[float]:
    """Frozen-core energy of each species (zero where nothing is frozen)."""
    out = []
    for a in range(len(hcore)):
        if frozen_core[a] == 0:
            out.append(0.0)
        elif not restricted[a] and len(fc_dm[a]) == 2:
            D0, D1 = fc_dm[a]
            out.append(0.5 * float(np.sum((D0 + D1) * hcore[a] + D0 * F_fc[a][0] + D1 * F_fc[a][1])))
        else:
            out.append(float(np.sum(fc_dm[a][0] * (hcore[a] + F_fc[a][0]))))
    return out
