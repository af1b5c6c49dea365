"""Electron-positron known answers of the reference, reproduced through the oracle.

The reference's quantum-positron tests run libint integrals and its multicomponent SCF; here the AO integrals
come from the oracle's McMurchie-Davidson code (s and p shells) and the SCF from its restatement of the
POLYQUANT_EPSCF fixed point, with the reference's own basis files (tests/golden/positron_bases.npz).  Pinned:
  * Li- + e+ SCF, tests/integration_tests/calculation/calculation_test.cpp:216-233 (1e-6; H_core(0,0) 1e-5);
  * the mixed-species CI elements on those orbitals, tests/unit_tests/ci/ci_test.cpp:578-673: HF diagonal
    -7.5257234633357024 (1e-6), every single excitation from HF zero (1e-6), the double {1,0,2,0} below 1e-3;
  * PsH natural spin orbitals, ci_test.cpp:873-892 (occupation sums 1e-8, coefficients 1e-6 / 1e-5).
"""
from types import SimpleNamespace

import numpy as np
import pytest

import oracle as O
from cases import li_wpos, psh_wpos
from polyquant_gb300.natural_orbitals import calculate_NOs

LOOSE, TIGHT = 1e-6, 1e-8  # POLYQUANT_TEST_EPSILON_LOOSE / _TIGHT


@pytest.fixture(scope="module")
def li():
    return li_wpos()


def test_li_wpos_scf(li):
    e, p = li["scf"]
    assert abs(li["E_scf"] - -7.5257234633) < LOOSE
    assert abs(e["E"] - -7.7455067859) < LOOSE and abs(p["E"] - 0.2197833078) < LOOSE
    assert abs(e["eps"][0][0] - -2.417238715) < LOOSE and abs(p["eps"][0][0] - -0.1098592288) < LOOSE
    assert abs(abs(e["C"][0][0, 0]) - 0.697239) < LOOSE and abs(abs(p["C"][0][0, 0]) - 0.000439523) < LOOSE
    assert abs(e["F"][0][0, 0] - -2.1305440797) < LOOSE and abs(p["F"][0][0, 0] - 11.5013794256) < LOOSE
    assert abs(e["D"][0][0, 0] - 0.494599) < LOOSE and abs(p["D"][0][0, 0] - 0.0000000154) < LOOSE
    assert abs(li["H_core"][0][0, 0] - -4.41628) < 10 * LOOSE and abs(li["H_core"][1][0, 0] - 15.602987) < LOOSE


def test_li_wpos_mixed_elements(li):
    d = O.Detset(li["problem"])
    I = d.lookup([0, 0, 0, 0])
    assert abs(d.slater_condon(I, I) - -7.5257234633357024) < LOOSE
    for slot in range(3):  # electron alpha, electron beta, positron alpha singles of HF: Brillouin
        s, sp = divmod(slot, 2)
        strings = d.strings(s, sp)
        n = 0
        for k in range(1, len(strings)):
            if O.num_excitation(strings[0], strings[k]) != 1:
                continue
            t = [0, 0, 0, 0]
            t[slot] = k
            assert abs(d.slater_condon(I, d.lookup(t))) < LOOSE
            n += 1
        assert n > 0
    assert abs(d.slater_condon(I, d.lookup([1, 0, 2, 0]))) < 1e-3


def test_psh_natural_spin_orbitals():
    r = psh_wpos()
    p = r["problem"]
    d = O.Detset(p)
    w, V = np.linalg.eigh(d.dense_ham())
    space = SimpleNamespace(n_species=2, n_orb=p.n_orb, n_alpha=p.n_alpha, n_beta=p.n_beta,
                            restricted=p.restricted, excitation_level=p.ex_level)
    no = calculate_NOs(space, None, [[r["C"][0]], [r["C"][1]]],
                       rdm1=lambda st, s, spin: d.create_1rdm(V[:, st], s, spin))
    assert abs(no["occ_nso"][0][0][0].sum() - 1.0) < TIGHT and abs(no["occ_nso"][0][1][0].sum() - 1.0) < TIGHT
    Ce, Cp = np.abs(no["C_nso"][0][0][0][:, 0]), np.abs(no["C_nso"][0][1][0][:, 0])
    assert np.abs(Ce - [0.300771, 0.345285, 0.43364, 0.0889083, 0.00747211]).max() < LOOSE
    assert abs(Cp[0] - 1.36173) < 10 * LOOSE and abs(Cp[1] - 0.428029) < LOOSE


def test_psh_multispecies_sigma_fast_vs_slow():
    """ci_test.cpp:770-852: PsH_wpos.json bases, excitation level (1,1,1) for both species, sigma of e0, e5 and
    the uniform vector by the pair-once builder equals the dense builder to 10 * 1e-14."""
    p = psh_wpos(ex=((1, 1, 1), (1, 1, 1)))["problem"]
    d = O.Detset(p)
    n = d.n_dets
    for C in (np.eye(n)[:, [0]], np.eye(n)[:, [5]], np.full((n, 1), 1.0 / n)):
        fast, slow = d.sigma(C), d.sigma(C, slow=True)
        assert np.abs(fast - slow).max() < 10 * 1e-14
