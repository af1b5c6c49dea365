"""Shared CI test cases (H2O/STO-3G from the oracle's integral code, seeded synthetics)."""
from __future__ import annotations

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
