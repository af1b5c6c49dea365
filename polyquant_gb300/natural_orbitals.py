"""Natural spin orbitals of CI states on top of the device 1-RDM.

Restates POLYQUANT_EPCI::calculate_NOs (src/ci/epci.cpp:200-318) and
diag_dm_helper (epci.cpp:130-146):

* for each requested state and species, the active-space 1-RDM of each spin
  (``pq_ci_rdm1`` on the device, create_1rdm in the reference) is placed in
  the full MO space at rows/columns [frozen_core, frozen_core + n_active), and
  the frozen-core orbitals get occupation 1 on the diagonal (fc_occ,
  epci.cpp:52-90);
* a species with one particle has only the alpha matrix; a restricted species
  with more than one particle takes its beta matrix from alpha
  (epci.cpp:235-237);
* the matrix is diagonalised, the occupations sorted in decreasing order with
  the eigenvectors permuted alike, and the natural spin orbitals expressed in
  the AO basis as C_nso = C_mo @ U (C_mo = the SCF orbitals, n_ao x n_mo);
* a species with no excitations (excitation level 0 for alpha and beta)
  keeps its SCF orbitals and occupations (epci.cpp:276-291).

The eigen-decomposition of an n_mo x n_mo matrix is host work, as in the
reference; the O(N_det) part, the 1-RDM, runs on the GPU.
"""
from __future__ import annotations

from typing import Callable, Optional, Sequence

import numpy as np


def diag_dm(dm: np.ndarray, transforming_orbs: np.ndarray):
    """(occupations in decreasing order, transforming_orbs @ eigenvectors in the same order) (epci.cpp:130-146)."""
    occ, U = np.linalg.eigh(dm)
    order = np.argsort(-occ, kind="stable")
    return occ[order], transforming_orbs @ U[:, order]


def calculate_NOs(ds, C_ci, C_combined: Sequence[Sequence[np.ndarray]], NO_states: Sequence[int] = (0,),
                  frozen_core: Optional[Sequence[int]] = None, excitation_level: Optional[Sequence[Sequence[int]]] = None,
                  occ_combined: Optional[Sequence[Sequence[np.ndarray]]] = None,
                  rdm1: Optional[Callable[[int, int, int], np.ndarray]] = None) -> dict:
    """Natural spin orbitals of the states ``NO_states`` of the CI vectors ``C_ci`` (N_dets x k, torch CUDA).

    ds                POLYQUANT_DETSET the vectors belong to (its n_species, n_orb = active orbitals,
                      n_alpha, n_beta, restricted and excitation_level per species are read).
    C_combined        [species][spin] SCF orbitals, n_ao x n_mo (one entry per spin block: 1 for restricted).
    frozen_core       frozen orbitals per species (default 0).
    excitation_level  [species][alpha, beta, total] as given to the determinant set (default: the set's own).
    occ_combined      [species][spin] SCF occupations, used for species without excitations
                      (default: aufbau, 1 per occupied spin orbital).
    rdm1              optional (state, species, spin) -> n_active x n_active density matrix; default: the
                      device 1-RDM of ds.

    Returns {"dm1", "C_nso", "occ_nso"}, each indexed [state_vec_idx][species][spin] like the reference's
    members of the same names.
    """
    ns = ds.n_species
    fc = list(frozen_core) if frozen_core is not None else [0] * ns
    n_act, n_a, n_b = list(ds.n_orb), list(ds.n_alpha), list(ds.n_beta)
    restricted = [bool(r) for r in ds.restricted]
    lv = excitation_level if excitation_level is not None else ds.excitation_level
    if rdm1 is None:
        def rdm1(state, sp, spin):
            return ds.rdm1(C_ci[:, state], spin=spin, species=sp)

    out = {"dm1": [], "C_nso": [], "occ_nso": []}
    for state in NO_states:
        dms, cs, occs = [], [], []
        for s in range(ns):
            blocks = C_combined[s]
            n_mo = blocks[0].shape[1]
            if n_mo < fc[s] + n_act[s]:
                raise ValueError(f"species {s}: {n_mo} MOs cannot hold {fc[s]} frozen + {n_act[s]} active orbitals")
            num_parts = n_a[s] + n_b[s] + 2 * fc[s]
            a0, a1 = fc[s], fc[s] + n_act[s]

            def full(spin):
                dm = np.zeros((n_mo, n_mo))
                dm[np.arange(fc[s]), np.arange(fc[s])] = 1.0
                dm[a0:a1, a0:a1] = rdm1(state, s, spin)
                return dm

            if num_parts > 1:
                d0 = full(0)
                d1 = full(1) if not restricted[s] else d0.copy()
                dm_s = [d0, d1]
            else:
                dm_s = [full(0)]
            dms.append(dm_s)
            no_exc = lv[s][0] == 0 and lv[s][1] == 0
            c_s, o_s = [], []
            for spin in range(len(dm_s)):
                C_mo = blocks[spin % len(blocks)] if not restricted[s] else blocks[0]
                if no_exc:
                    if occ_combined is not None:
                        occ = np.asarray(occ_combined[s][spin % len(occ_combined[s])], dtype=float)
                    else:
                        occ = np.zeros(n_mo)
                        occ[: fc[s] + (n_a[s] if spin == 0 else n_b[s])] = 1.0
                    c_s.append(np.array(C_mo, dtype=float))
                    o_s.append(occ)
                else:
                    occ, C = diag_dm(dm_s[spin], C_mo)
                    c_s.append(C)
                    o_s.append(occ)
            cs.append(c_s)
            occs.append(o_s)
        out["dm1"].append(dms)
        out["C_nso"].append(cs)
        out["occ_nso"].append(occs)
    return out
