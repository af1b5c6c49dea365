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


def _oracle_solver(p):
    """A selected space solved on the host: the oracle's dense H (the reference's Slater-Condon rules)
    restricted to the selected determinants, in the library's order (full product of the lists, species 0
    alpha outermost)."""
    import oracle as O

    ref = O.Detset(p)
    H = ref.dense_ham()
    ns = len(p.n_orb)
    pos = [[{int(m): i for i, m in enumerate(ref.strings(s, sp)[:, -1])} for sp in range(2)] for s in range(ns)]
    fidx = {tuple(t): i for i, t in enumerate(ref.unfold())}

    def solve(strings):
        lists = [strings[s][sp] for s in range(ns) for sp in range(2)]
        unfold = np.array(list(itertools.product(*[range(len(l)) for l in lists])), dtype=np.int32)
        idx = [fidx[tuple(pos[k // 2][k % 2][lists[k][t[k]]] for k in range(2 * ns))] for t in unfold]
        w, v = np.linalg.eigh(H[np.ix_(idx, idx)])
        return w[:1], v[:, 0], unfold

    return solve, np.linalg.eigvalsh(H)[0], ref.n_dets


def test_nested_selection_is_monotone_and_reaches_the_full_space():
    """The driver's selection on the host (oracle solver): energies never rise along decreasing thresholds,
    the loosest threshold keeps a proper subspace, eps = 0 selects every string and gives the full-space
    ground state."""
    from cases import batch_dict, synthetic_fci
    from polyquant_gb300.heatbath import heat_bath_ci

    for p in (synthetic_fci(7, 2, 2, seed=3), synthetic_ep(6, 1, 1, 5, 1, 0, seed=2)):
        d = batch_dict(p)
        prob = {k: d[k] for k in ("n_orb", "n_alpha", "n_beta", "h1", "eri", "restricted", "charge")}
        solve, e_full, n_full = _oracle_solver(p)
        recs = heat_bath_ci(prob, [0.1, 1e-2, 1e-3, 0.0], solver=solve)
        es = [r["energies"][0] for r in recs]
        assert all(b <= a + 1e-12 for a, b in zip(es, es[1:])), es
        assert recs[0]["n_dets"] < n_full and recs[-1]["n_dets"] == n_full
        assert abs(es[-1] - e_full) < 1e-10
        sizes = [r["n_strings"] for r in recs]
        for a, b in zip(sizes, sizes[1:]):
            assert all(b[s][sp] >= a[s][sp] for s in range(len(a)) for sp in range(2))
