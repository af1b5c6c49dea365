"""Natural spin orbitals (calculate_NOs, src/ci/epci.cpp:200-318; diag_dm_helper, epci.cpp:130-146).

The host assembly (frozen-core embedding, spin handling, sorting, rotation to the AO basis) is checked on the
CPU with the oracle's create_1rdm standing in for the device 1-RDM, against the reference's own golden data:
H- in its five-shell s basis, CISD [1,1,2], state 0, compared with pyscf natural orbitals
(tests/unit_tests/ci/ci_test.cpp:854-871: occupations of one spin = spin-summed / 2 within 1e-6,
|C_NO| within 1e-3)."""
from types import SimpleNamespace

import numpy as np
import pytest

import oracle as O
from cases import h_minus, synthetic_ep, synthetic_fci
from polyquant_gb300.natural_orbitals import calculate_NOs

OCC_TOL = 1e-6   # POLYQUANT_TEST_EPSILON_LOOSE in the reference test
NO_TOL = 1e-3


def space(p):
    return SimpleNamespace(n_species=p.n_species, n_orb=p.n_orb, n_alpha=p.n_alpha, n_beta=p.n_beta,
                           restricted=p.restricted, excitation_level=p.ex_level)


def oracle_rdm(d, V):
    return lambda state, sp, spin: d.create_1rdm(V[:, state], sp, spin)


@pytest.fixture(scope="module")
def hm():
    r = h_minus()
    d = O.Detset(r["problem"])
    w, V = np.linalg.eigh(d.dense_ham())
    return r, d, w, V


def test_h_minus_natural_orbitals_match_reference_data(hm):
    r, d, w, V = hm
    no = calculate_NOs(space(r["problem"]), None, [[r["C"]]], NO_states=[0], rdm1=oracle_rdm(d, V))
    occ = no["occ_nso"][0][0]
    C = no["C_nso"][0][0]
    assert len(occ) == 2 and len(C) == 2          # two electrons: alpha and beta matrices
    assert np.abs(occ[0] - r["no_occ"] / 2).max() < OCC_TOL
    assert np.abs(np.abs(C[0]) - np.abs(r["no_ao"])).max() < NO_TOL
    # restricted: beta copies alpha
    assert np.array_equal(no["dm1"][0][0][1], no["dm1"][0][0][0])
    # natural orbitals are S-orthonormal and the occupations sum to the electron count of one spin
    assert np.abs(C[0].T @ r["S"] @ C[0] - np.eye(5)).max() < 1e-10
    assert abs(occ[0].sum() - 1.0) < 1e-12
    assert np.all(np.diff(occ[0]) <= 0)


def test_frozen_core_embedding_and_states():
    p = synthetic_fci(6, 2, 2, seed=11)
    d = O.Detset(p)
    w, V = np.linalg.eigh(d.dense_ham())
    fc, dv = 2, 1
    n_mo = fc + 6 + dv
    Cmo = np.linalg.qr(np.random.default_rng(3).standard_normal((n_mo, n_mo)))[0]
    no = calculate_NOs(space(p), None, [[Cmo]], NO_states=[0, 2], frozen_core=[fc], rdm1=oracle_rdm(d, V))
    assert len(no["dm1"]) == 2
    for k, state in enumerate((0, 2)):
        dm = no["dm1"][k][0][0]
        assert np.array_equal(dm[:fc, :fc], np.eye(fc))
        assert np.abs(dm[:fc, fc:]).max() == 0 and np.abs(dm[fc + 6:, :]).max() == 0
        assert np.abs(dm[fc:fc + 6, fc:fc + 6] - d.create_1rdm(V[:, state], 0, 0)).max() < 1e-14
        occ, C = no["occ_nso"][k][0][0], no["C_nso"][k][0][0]
        assert abs(occ.sum() - (fc + 2)) < 1e-12
        assert np.abs(occ[:fc] - 1.0).max() < 1e-12
        # C_nso diagonalises the density matrix expressed in the rotated basis
        U = Cmo.T @ C
        assert np.abs(U.T @ dm @ U - np.diag(occ)).max() < 1e-12


def test_electron_positron_species():
    # 2 electrons (restricted) + 1 positron (one particle: alpha matrix only)
    p = synthetic_ep(5, 1, 1, 4, 1, 0, seed=5)
    d = O.Detset(p)
    w, V = np.linalg.eigh(d.dense_ham())
    Ce, Cp = np.eye(5), np.eye(4)
    no = calculate_NOs(space(p), None, [[Ce], [Cp]], rdm1=oracle_rdm(d, V))
    e_occ, p_occ = no["occ_nso"][0]
    assert len(e_occ) == 2 and len(p_occ) == 1
    assert abs(e_occ[0].sum() - 1.0) < 1e-12 and abs(p_occ[0].sum() - 1.0) < 1e-12
    assert np.abs(no["dm1"][0][1][0] - d.create_1rdm(V[:, 0], 1, 0)).max() < 1e-14


def test_species_without_excitations_keeps_scf_orbitals():
    # positron frozen in its SCF orbital: excitation level 0 for both spins
    p = synthetic_ep(5, 1, 1, 4, 1, 0, seed=6, ex_p=[0, 0, 0])
    d = O.Detset(p)
    w, V = np.linalg.eigh(d.dense_ham())
    Cp = np.linalg.qr(np.random.default_rng(1).standard_normal((4, 4)))[0]
    no = calculate_NOs(space(p), None, [[np.eye(5)], [Cp]], rdm1=oracle_rdm(d, V))
    assert np.array_equal(no["C_nso"][0][1][0], Cp)
    assert np.array_equal(no["occ_nso"][0][1][0], np.array([1.0, 0, 0, 0]))
