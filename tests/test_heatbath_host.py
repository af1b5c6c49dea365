"""Host parts of the heat-bath string selection (polyquant_gb300/heatbath.py, an extension): the
excitation enumeration of a string against brute force, and the excitation bounds against the integral
blocks they are taken from."""
import itertools

import numpy as np

from cases import synthetic_ep
from polyquant_gb300.heatbath import excitation_bounds, string_excitations


def test_string_excitations_match_brute_force():
    n, m = 7, 0b0101101
    singles, doubles = string_excitations(m, n)
    occ = [o for o in range(n) if (m >> o) & 1]
    all_strings = [sum(1 << i for i in c) for c in itertools.combinations(range(n), len(occ))]
    one = {x for x in all_strings if bin(x ^ m).count("1") == 2}
    two = {x for x in all_strings if bin(x ^ m).count("1") == 4}
    assert {J for (_, _, J) in singles} == one and len(singles) == len(one)
    assert {J for (*_, J) in doubles} == two and len(doubles) == len(two)
    for h, p, J in singles:
        assert (m >> h) & 1 and not (m >> p) & 1 and J == m ^ (1 << h) ^ (1 << p)
    for h1, h2, p1, p2, J in doubles:
        assert h1 < h2 and p1 < p2 and J == m ^ (1 << h1) ^ (1 << h2) ^ (1 << p1) ^ (1 << p2)


def test_excitation_bounds_cover_every_partner_block():
    p = synthetic_ep(5, 2, 1, 4, 1, 1, seed=3)
    U, E = excitation_bounds(p.n_orb, p.h1, p.eri, p.restricted)
    ee, pp, ep = p.eri[(0, 0, 0, 0)], p.eri[(1, 0, 1, 0)], p.eri[(0, 0, 1, 0)]
    # electron pairs: partners are the other electron spin (ee) and both positron spins (ep)
    want_e = np.maximum(np.abs(ee).max(axis=1), np.abs(ep).max(axis=1))
    assert np.allclose(U[0][0], want_e) and np.allclose(U[0][1], want_e)
    want_p = np.maximum(np.abs(pp).max(axis=1), np.abs(ep.T).max(axis=1))
    assert np.allclose(U[1][0], want_p)
    assert np.array_equal(E[0][0], ee) and np.array_equal(E[1][1], pp)
