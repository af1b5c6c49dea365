"""Frozen-core operator and energy (calculate_frozen_core_ints, src/integral/integral.cpp:64-95, 569-699;
frozen-core energy, src/ci/epci.cpp:110-128) checked by an exact identity: the active-space CI on
C_act^T F_fc C_act with the energy shifted by E_fc has the spectrum of the full-space Hamiltonian restricted to
the determinants whose frozen orbitals are doubly occupied."""
import numpy as np

import oracle as O
from cases import h2o_problem, li_wpos
from polyquant_gb300.frozen_core import calculate_frozen_core_ints, frozen_core_density, frozen_core_energy


def frozen_block_spectrum(d, frozen_slots, n_fc):
    """Eigenvalues of the full-space H over determinants whose listed string slots hold orbitals 0..n_fc-1."""
    keep_mask = (1 << n_fc) - 1
    u = d.unfold()
    masks = {}
    ok = np.ones(d.n_dets, dtype=bool)
    for slot in frozen_slots:
        s, sp = divmod(slot, 2)
        if (s, sp) not in masks:
            masks[(s, sp)] = np.array([int(w[-1]) for w in d.strings(s, sp)], dtype=object)
        ok &= np.array([(int(masks[(s, sp)][i]) & keep_mask) == keep_mask for i in u[:, slot]])
    H = d.dense_ham()
    return np.linalg.eigvalsh(H[np.ix_(ok, ok)]), int(ok.sum())


def test_h2o_frozen_1s(h2o):
    r = h2o("file")
    C, T, V, eri = r["C"], r["T"], r["V"], r["eri"]
    full = O.Detset(h2o_problem(r, [2, 2, 4]))
    w_full, n_kept = frozen_block_spectrum(full, [0, 1], 1)
    Dfc = frozen_core_density(C, 1)
    F = calculate_frozen_core_ints([T + V], [[Dfc]], [1], {(0, 0): eri}, [-1.0], [True])
    E_fc = frozen_core_energy([T + V], [[Dfc]], F, [1], [True])[0]
    Ca = C[:, 1:]
    h = Ca.T @ F[0][0] @ Ca
    act = O.Detset(O.CIProblem([6], [4], [4], [[h, h]], {(0, 0, 0, 0): O.ao2mo_full(eri, Ca, Ca)}, [[2, 2, 4]],
                               restricted=[1], charge=[-1.0]))
    assert act.n_dets == n_kept == 225
    w_act = np.linalg.eigvalsh(act.dense_ham()) + E_fc
    assert np.abs(w_act - w_full).max() < 1e-9
    # E_fc is the closed-shell energy of the frozen orbital: 2 h_00 + (00|00) in the MO basis
    c0 = C[:, 0]
    j00 = np.einsum("ijkl,i,j,k,l->", eri, c0, c0, c0, c0)
    assert abs(E_fc - (2 * c0 @ (T + V) @ c0 + j00)) < 1e-12


def test_li_wpos_frozen_electron_core():
    r = li_wpos()
    p = r["problem"]
    full = O.Detset(p)
    w_full, n_kept = frozen_block_spectrum(full, [0, 1], 1)
    He, Hp = r["H_core"]
    ao = r["ao"]
    Ce, Cp = r["C"]
    Dfc = frozen_core_density(Ce, 1)
    F = calculate_frozen_core_ints([He, Hp], [[Dfc], [np.zeros_like(Hp)]], [1, 0],
                                   {(0, 0): ao["eri_e"], (1, 1): ao["eri_p"], (0, 1): ao["eri_ep"]}, [-1.0, 1.0], [True, False])
    E_fc = frozen_core_energy([He, Hp], [[Dfc], [np.zeros_like(Hp)]], F, [1, 0], [True, False])
    assert E_fc[1] == 0.0
    Ca = Ce[:, 1:]
    he = Ca.T @ F[0][0] @ Ca
    hp = Cp.T @ F[1][0] @ Cp
    eri_act = {(0, 0, 0, 0): O.ao2mo_full(ao["eri_e"], Ca, Ca), (1, 0, 1, 0): O.ao2mo_full(ao["eri_p"], Cp, Cp),
               (0, 0, 1, 0): O.ao2mo_full(ao["eri_ep"], Ca, Cp)}
    act = O.Detset(O.CIProblem([15, 16], [1, 1], [1, 0], [[he, he], [hp, hp]], eri_act, [[1, 1, 1], [1, 1, 1]],
                               restricted=[1, 1], charge=[-1.0, 1.0]))
    assert act.n_dets == n_kept
    w_act = np.linalg.eigvalsh(act.dense_ham()) + E_fc[0]
    assert np.abs(w_act - w_full).max() < 1e-9


def test_frozen_core_energy_reference_value(h2o):
    """tests/unit_tests/ci/ci_test.cpp:132-146: H2O/STO-3G (file basis), two frozen orbitals,
    frozen_core_energy = -71.3745646924 (1e-6)."""
    r = h2o("file")
    C, T, V, eri = r["C"], r["T"], r["V"], r["eri"]
    Dfc = frozen_core_density(C, 2)
    F = calculate_frozen_core_ints([T + V], [[Dfc]], [2], {(0, 0): eri}, [-1.0], [True])
    assert abs(frozen_core_energy([T + V], [[Dfc]], F, [2], [True])[0] - -71.3745646924) < 1e-6
    # nothing frozen: zero, as ci_test.cpp:148-163 requires
    assert frozen_core_energy([T + V], [[0 * Dfc]], F, [0], [True]) == [0.0]


def test_unrestricted_frozen_core_with_a_nucleus_species():
    """Quantum-proton water (protons species 0, UHF electrons species 1), electron 1s-like orbital frozen in
    both spin blocks.  The reference's operator adds the electrons' frozen Coulomb field to the proton operator
    once per electron spin block; the single-count operator satisfies the frozen-block identity."""
    from cases import quantum_h_water

    qh = quantum_h_water()
    full = O.Detset(qh["problem"])
    w_full, n_kept = frozen_block_spectrum(full, [2, 3], 1)
    n, e = qh["scf"]
    (Hn, He), eri = qh["H_core"], qh["eri"]
    Cn, (Ca, Cb) = n["C"][0], e["C"]
    fc_dm = [[np.zeros_like(Hn)], [frozen_core_density(Ca, 1), frozen_core_density(Cb, 1)]]
    eris = {(0, 0): eri, (1, 1): eri, (0, 1): eri}
    F_ref = calculate_frozen_core_ints([Hn, He], fc_dm, [0, 1], eris, [1.0, -1.0], [True, False])
    F = calculate_frozen_core_ints([Hn, He], fc_dm, [0, 1], eris, [1.0, -1.0], [True, False],
                                   single_count_cross=True)
    cross = -np.einsum("ijkl,kl->ij", eri, fc_dm[1][0] + fc_dm[1][1])
    assert np.abs(F_ref[0][0] - F[0][0] - cross).max() < 1e-12
    assert all(np.array_equal(F_ref[1][s], F[1][s]) for s in range(2))
    E_fc = frozen_core_energy([Hn, He], fc_dm, F, [0, 1], [True, False])
    assert E_fc[0] == 0.0
    Ca_, Cb_ = Ca[:, 1:], Cb[:, 1:]
    mo = O.ao2mo_full
    eri_act = {(0, 0, 0, 0): mo(eri, Cn, Cn), (1, 0, 1, 0): mo(eri, Ca_, Ca_), (1, 1, 1, 1): mo(eri, Cb_, Cb_),
               (1, 0, 1, 1): mo(eri, Ca_, Cb_), (1, 1, 1, 0): mo(eri, Cb_, Ca_),
               (0, 0, 1, 0): mo(eri, Cn, Ca_), (0, 0, 1, 1): mo(eri, Cn, Cb_)}
    hn = Cn.T @ F[0][0] @ Cn
    act = O.Detset(O.CIProblem([7, 6], [1, 4], [1, 4], [[hn, hn], [Ca_.T @ F[1][0] @ Ca_, Cb_.T @ F[1][1] @ Cb_]],
                               eri_act, [[1, 1, 1], [1, 1, 1]], restricted=[1, 0], charge=[1.0, -1.0]))
    assert act.n_dets == n_kept
    w_act = np.linalg.eigvalsh(act.dense_ham()) + E_fc[1]
    assert np.abs(w_act - w_full).max() < 1e-9
