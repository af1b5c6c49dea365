"""Electron-nucleus known answers: H2O/STO-3G with both protons quantum
(tests/data/h2o_sto3g_quantumH{file,library}/h2o.json, tests/integration_tests/calculation/calculation_test.cpp:174-213),
reproduced through the oracle's integral code and multicomponent SCF, then the CI path on that system.

The reference's SCF adds the Coulomb term of an unrestricted partner species (here the electrons, 5a5b) once
per spin block in the Fock matrix of the other species; its test values carry that, and the restatement
reproduces them only with the same count (without it the total energy moves by 5.5 Eh).  The CI elements count
the cross term once (slater_condon_mixedparticle.cpp), so the CI HF diagonal is the single-count HF energy of
the same orbitals, which the last test checks independently in the AO basis."""
import numpy as np
import pytest

import oracle as O
from cases import quantum_h_water

LOOSE = 1e-6


@pytest.fixture(scope="module")
def qh():
    return quantum_h_water()


@pytest.mark.parametrize("basis", ["file", "library"])
def test_quantum_proton_scf(basis):
    """calculation_test.cpp:174-213: the same values for the file and the library STO-3G digits."""
    qh = quantum_h_water(basis=basis)
    n, e = qh["scf"]
    assert abs(qh["E_scf"] - -78.1165107917) < LOOSE
    assert abs(n["E"] - 3.0365625787) < LOOSE and abs(e["E"] - -81.1530733704) < LOOSE
    assert abs(n["eps"][0][0] - -6.7850710986) < LOOSE and abs(e["eps"][0][0] - -20.4054374486) < LOOSE
    assert abs(abs(n["C"][0][0, 0]) - 0.0384832) < LOOSE and abs(abs(e["C"][0][0, 0]) - 0.00598694) < LOOSE
    assert abs(n["F"][0][0, 0] - -4.3143) < LOOSE and abs(e["F"][0][0, 0] - 0.181054) < LOOSE
    assert abs(n["D"][0][0, 0] - 0.00148096) < LOOSE and abs(e["D"][0][0, 0] - 0.00646869) < LOOSE
    assert abs(qh["H_core"][0][0, 0] - 5.01601) < 10 * LOOSE and abs(qh["H_core"][1][0, 0] - -3.50184) < 10 * LOOSE


def test_ci_on_quantum_protons(qh):
    p = qh["problem"]
    d = O.Detset(p)
    rng = np.random.default_rng(0)
    C = rng.standard_normal((d.n_dets, 2))
    fast, slow = d.sigma(C), d.sigma(C, slow=True)
    H = d.dense_ham()
    scale = np.abs(slow).max()
    assert np.abs(fast - slow).max() < 1e-12 * scale and np.abs(fast - H @ C).max() < 1e-12 * scale
    assert np.abs(H - H.T).max() < 1e-12
    # HF diagonal = the single-count HF energy of the SCF orbitals, from AO densities
    n, e = qh["scf"]
    eri, (Hn, He) = qh["eri"], qh["H_core"]

    def J(D):
        return np.einsum("pqrs,rs->pq", eri, D)

    def K(D):
        return np.einsum("prqs,rs->pq", eri, D)

    Dn = 2 * n["D"][0]
    Da, Db = e["D"]
    De = Da + Db
    E_n = np.sum(Dn * Hn) + 0.5 * np.sum(Dn * J(Dn)) - np.sum(n["D"][0] * K(n["D"][0]))
    E_e = np.sum(De * He) + 0.5 * np.sum(De * J(De)) - 0.5 * (np.sum(Da * K(Da)) + np.sum(Db * K(Db)))
    E_ne = -np.sum(Dn * J(De))
    hf = d.lookup([0, 0, 0, 0])
    assert abs(d.diagonal()[hf] - (E_n + E_e + E_ne)) < 1e-9
    # and it differs from the reference's SCF energy by the second count of the cross term
    assert abs((E_n + E_e + E_ne) - (qh["E_scf"] - 0.5 * E_ne)) < 1e-6
