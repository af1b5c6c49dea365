"""Shared CI test cases (H2O/STO-3G from the oracle's integral code, seeded synthetics)."""
from __future__ import annotations

import functools

import numpy as np

import oracle as O
from polyquant_gb300 import synthetic


def h2o_problem(r, ex, n_alpha=5, n_beta=5):
    C = r["C"]
    n = C.shape[1]
    h = C.T @ (r["T"] + r["V"]) @ C
    eri = O.ao2mo_full(r["eri"], C, C)
    return O.CIProblem([n], [n_alpha], [n_beta], [[h, h]], {(0, 0, 0, 0): eri}, [ex], restricted=[1],
                       charge=[-1.0], e_const=r["e_nuc"])


def synthetic_fci(n, na, nb, seed=0, ex=None):
    h, eri = synthetic.fci_integrals(n, seed)
    if ex is None:
        ex = [na, nb, na + nb]
        ex = [min(na, n - na), min(nb, n - nb), min(na, n - na) + min(nb, n - nb)]
    return O.CIProblem([n], [na], [nb], [[h, h]], {(0, 0, 0, 0): eri}, [ex], restricted=[1], charge=[-1.0])


def synthetic_unrestricted(n, na, nb, seed=0, ex=None):
    """Different alpha/beta integrals (UHF-like spin blocks)."""
    ha, eaa = synthetic.fci_integrals(n, seed)
    hb, ebb = synthetic.fci_integrals(n, seed + 1)
    rng = np.random.default_rng(seed + 2)
    eab = 0.5 * (eaa + ebb) + 0.01 * rng.standard_normal(eaa.shape)
    if ex is None:
        ex = [min(na, n - na), min(nb, n - nb), min(na, n - na) + min(nb, n - nb)]
    return O.CIProblem([n], [na], [nb], [[ha, hb]],
                       {(0, 0, 0, 0): eaa, (0, 1, 0, 1): ebb, (0, 0, 0, 1): eab, (0, 1, 0, 0): eab.T},
                       [ex], restricted=[0], charge=[-1.0])


def synthetic_ep(n_e, ne_a, ne_b, n_p, np_a, np_b, seed=0, ex_e=None, ex_p=None, max_coll=2 ** 31 - 1):
    """Electron + positron problem (positron charge +1, electrons -1)."""
    h_e, h_p, ee, pp, ep = synthetic.ep_integrals(n_e, n_p, seed)
    if ex_e is None:
        ex_e = [min(ne_a, n_e - ne_a), min(ne_b, n_e - ne_b), min(ne_a, n_e - ne_a) + min(ne_b, n_e - ne_b)]
    if ex_p is None:
        ex_p = [min(np_a, n_p - np_a), min(np_b, n_p - np_b), min(np_a, n_p - np_a) + min(np_b, n_p - np_b)]
    return O.CIProblem([n_e, n_p], [ne_a, np_a], [ne_b, np_b], [[h_e, h_e], [h_p, h_p]],
                       {(0, 0, 0, 0): ee, (1, 0, 1, 0): pp, (0, 0, 1, 0): ep},
                       [ex_e, ex_p], restricted=[1, 1], charge=[-1.0, 1.0], max_collective=max_coll)


def synthetic_en(n_e, ne_a, ne_b, n_n, nn_a, nn_b, seed=0, nuc_charge=2.0):
    """Electrons + a quantum-nucleus species with unrestricted (different alpha and beta) integral blocks and
    charge ``nuc_charge``: cross-species terms carry charge[0] * charge[1] = -nuc_charge, and the nuclear
    alpha-alpha, beta-beta, alpha-beta and electron-nucleus blocks are all distinct."""
    h_e, h_na, ee, nna, en_a = synthetic.ep_integrals(n_e, n_n, seed)
    _, h_nb, _, nnb, en_b = synthetic.ep_integrals(n_e, n_n, seed + 1)
    nn_ab = 0.5 * (nna + nnb)
    ex_e = [min(ne_a, n_e - ne_a), min(ne_b, n_e - ne_b), min(ne_a, n_e - ne_a) + min(ne_b, n_e - ne_b)]
    ex_n = [min(nn_a, n_n - nn_a), min(nn_b, n_n - nn_b), min(nn_a, n_n - nn_a) + min(nn_b, n_n - nn_b)]
    eri = {(0, 0, 0, 0): ee, (1, 0, 1, 0): nna, (1, 1, 1, 1): nnb, (1, 0, 1, 1): nn_ab, (1, 1, 1, 0): nn_ab.T,
           (0, 0, 1, 0): en_a, (0, 0, 1, 1): en_b}
    return O.CIProblem([n_e, n_n], [ne_a, nn_a], [ne_b, nn_b], [[h_e, h_e], [h_na, h_nb]], eri, [ex_e, ex_n],
                       restricted=[1, 0], charge=[-1.0, nuc_charge])


def batch_dict(p):
    """CIProblem -> keyword dict of CIBatch / POLYQUANT_DETSET."""
    return dict(n_orb=p.n_orb, n_alpha=p.n_alpha, n_beta=p.n_beta, h1=p.h1, eri=p.eri, excitation_level=p.ex_level,
                restricted=p.restricted, charge=p.charge, max_collective_excitation_level=p.max_collective)


def h_minus():
    """H- in the reference's five-shell s basis (golden fixture h_minus_no_golden.npz): AO integrals and RHF
    from the oracle's Gaussian-integral code, MO integrals, and the CISD [1,1,2] problem of
    tests/data/PsH_wpos/H_minus.json."""
    import os

    import gaussian_ints as G

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "h_minus_no_golden.npz"))
    shells = [("s", list(g["shell_exp"][i, :n]), list(g["shell_coef"][i, :n])) for i, n in enumerate(g["shell_nprim"])]
    mol = G.Molecule(["H"], [0.0, 0.0, 0.0], {"H": shells})
    S, T, V = mol.one_body()
    eri = mol.eri()
    E, C, eps = G.rhf(S, T + V, eri, 1, mol.e_nuc())
    h = C.T @ (T + V) @ C
    p = O.CIProblem([C.shape[1]], [1], [1], [[h, h]], {(0, 0, 0, 0): O.ao2mo_full(eri, C, C)}, [[1, 1, 2]],
                    restricted=[1], charge=[-1.0], e_const=mol.e_nuc())
    return dict(problem=p, C=C, S=S, E_rhf=E, no_occ=g["no_occ"], no_ao=g["no_ao"])


def _shells(g, prefix):
    return [("s" if g[prefix + "_kind"][i] == 0 else "p", list(g[prefix + "_exp"][i, :n]),
             list(g[prefix + "_coef"][i, :n])) for i, n in enumerate(g[prefix + "_nprim"])]


def ep_atom(symbol, e_shells, p_shells, n_e_alpha, n_e_beta, ex, max_coll=2 ** 31 - 1):
    """One atom at the origin with electrons (restricted) and one positron (charge +1, mass 1): AO integrals
    from the oracle's Gaussian-integral code, the multicomponent SCF, and the CI problem in the MO basis
    (h = C^T (T - qV) C, integral.cpp:166-205; (ij|kl) blocks as calculate_mo_2_body_integrals fills them)."""
    import gaussian_ints as G

    me = G.Molecule([symbol], [0.0, 0.0, 0.0], {symbol: e_shells})
    mp = G.Molecule([symbol], [0.0, 0.0, 0.0], {symbol: p_shells})
    Se, Te, Ve = me.one_body()
    Sp, Tp, Vp = mp.one_body()
    eri_e = me.eri()
    eri_p = eri_e if p_shells == e_shells else mp.eri()
    eri_ep = eri_e if p_shells == e_shells else me.eri_with(mp)
    He, Hp = Te + Ve, Tp - Vp   # T/mass - q V with q = -1 (electrons), +1 (positron), mass 1
    spec = [dict(S=Se, H=He, eri=eri_e, n_alpha=n_e_alpha, n_beta=n_e_beta, restricted=True, charge=-1.0),
            dict(S=Sp, H=Hp, eri=eri_p, n_alpha=1, n_beta=0, restricted=False, charge=1.0)]
    E, res = G.epscf(spec, {(0, 1): eri_ep}, e_nuc=me.e_nuc())
    Ce, Cp = res[0]["C"][0], res[1]["C"][0]
    he, hp = Ce.T @ He @ Ce, Cp.T @ Hp @ Cp
    eri = {(0, 0, 0, 0): O.ao2mo_full(eri_e, Ce, Ce), (1, 0, 1, 0): O.ao2mo_full(eri_p, Cp, Cp),
           (0, 0, 1, 0): O.ao2mo_full(eri_ep, Ce, Cp)}
    p = O.CIProblem([Ce.shape[1], Cp.shape[1]], [n_e_alpha, 1], [n_e_beta, 0], [[he, he], [hp, hp]], eri, ex,
                    restricted=[1, 1], charge=[-1.0, 1.0], max_collective=max_coll, e_const=me.e_nuc())
    return dict(problem=p, E_scf=E, scf=res, H_core=[He, Hp], C=[Ce, Cp],
                ao=dict(eri_e=eri_e, eri_p=eri_p, eri_ep=eri_ep))


@functools.lru_cache(maxsize=None)
def li_wpos(ex=((1, 1, 1), (1, 1, 1))):
    """Li- + e+ in the reference's Li_basis.g94 for both species (tests/data/li-_custombasis_wpos/Li_wpos.json)."""
    import os

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "positron_bases.npz"))
    sh = _shells(g, "li")
    return ep_atom("Li", sh, sh, 2, 2, [list(e) for e in ex])


@functools.lru_cache(maxsize=None)
def psh_wpos(ex=((1, 1, 1), (1, 0, 1))):
    """PsH: H, two electrons and a positron in the bases of tests/data/PsH_wpos/PsH_wpos_CI.json."""
    import os

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "positron_bases.npz"))
    return ep_atom("H", _shells(g, "psh_e"), _shells(g, "psh_p"), 1, 1, [list(e) for e in ex])


@functools.lru_cache(maxsize=None)
def quantum_h_water(ex_n=(1, 1, 1), ex_e=(1, 1, 1), basis="file"):
    """H2O/STO-3G with both protons quantum (tests/data/h2o_sto3g_quantumH{file,library}/h2o.json, ``basis`` the
    file or library STO-3G digits): species 0 = the two
    protons (mass 1.00782503223, charge +1, restricted 1a1b; the reference orders species by name and "H"
    sorts before "electron"), species 1 = the ten electrons (unrestricted 5a5b), both in the STO-3G basis on all
    three centres; only the oxygen nucleus is a classical charge.  SCF through the oracle's multicomponent
    restatement with the reference's per-spin-block cross-species Coulomb count; CI problem in the MO basis
    with separate electron alpha and beta orbitals."""
    import gaussian_ints as G

    mol = G.Molecule(G.H2O_SYMBOLS, G.H2O_GEOMETRY, basis)
    S, T, V = mol.one_body(nuclear_charges={"H": 0.0, "O": 8.0})
    eri = mol.eri()
    m_h = 1.00782503223
    Hn, He = T / m_h - V, T + V
    spec = [dict(S=S, H=Hn, eri=eri, n_alpha=1, n_beta=1, restricted=True, charge=1.0),
            dict(S=S, H=He, eri=eri, n_alpha=5, n_beta=5, restricted=False, charge=-1.0)]
    E, res = G.epscf(spec, {(0, 1): eri}, e_nuc=0.0, cross_repeat_unrestricted=True)
    Cn = res[0]["C"][0]
    Ca, Cb = res[1]["C"]
    h_n = Cn.T @ Hn @ Cn
    h_a, h_b = Ca.T @ He @ Ca, Cb.T @ He @ Cb
    mo = O.ao2mo_full
    eri_mo = {(0, 0, 0, 0): mo(eri, Cn, Cn),
              (1, 0, 1, 0): mo(eri, Ca, Ca), (1, 1, 1, 1): mo(eri, Cb, Cb),
              (1, 0, 1, 1): mo(eri, Ca, Cb), (1, 1, 1, 0): mo(eri, Cb, Ca),
              (0, 0, 1, 0): mo(eri, Cn, Ca), (0, 0, 1, 1): mo(eri, Cn, Cb)}
    p = O.CIProblem([7, 7], [1, 5], [1, 5], [[h_n, h_n], [h_a, h_b]], eri_mo, [list(ex_n), list(ex_e)],
                    restricted=[1, 0], charge=[1.0, -1.0])
    return dict(problem=p, E_scf=E, scf=res, H_core=[Hn, He], S=S, eri=eri)
