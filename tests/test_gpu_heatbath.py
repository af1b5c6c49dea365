"""Heat-bath selection over strings (polyquant_gb300/heatbath.py, an extension with no reference
counterpart) on the GPU: nested selections give non-increasing variational energies that reach the
full-product energy at eps = 0, and a selected space's sigma and lowest root agree with the oracle's dense
Hamiltonian restricted to the selected determinants (the oracle restates the reference's Slater-Condon
rules, slater_condon_singleparticle.cpp / slater_condon_mixedparticle.cpp)."""
import numpy as np
import pytest

import oracle as O
from cases import batch_dict, synthetic_ep, synthetic_fci

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = {
    "ep_10o_1a1b_x_8o_1p": (lambda: synthetic_ep(10, 1, 1, 8, 1, 0, seed=5), [0.1, 1e-2, 1e-3, 1e-4, 0.0]),
    "fci_9o_3a3b": (lambda: synthetic_fci(9, 3, 3, seed=6), [0.05, 5e-3, 5e-4, 0.0]),
}


def _problem(p):
    d = batch_dict(p)
    return {k: d[k] for k in ("n_orb", "n_alpha", "n_beta", "h1", "eri", "restricted", "charge")}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    from polyquant_gb300.detset import POLYQUANT_DETSET
    from polyquant_gb300.heatbath import heat_bath_ci

    make, eps = CASES[request.param]
    p = make()
    recs = heat_bath_ci(_problem(p), eps, convergence_E=1e-10)
    full = POLYQUANT_DETSET(**batch_dict(p))
    e_full, info = full.davidson(num_states=1, num_subspace_vec=8, convergence_E=1e-10)
    assert info["converged"]
    yield request.param, p, recs, full, e_full[0]
    full.close()


def test_energies_monotone_and_reach_full_product(case):
    name, p, recs, full, e_full = case
    es = [r["energies"][0] for r in recs]
    for a, b in zip(es, es[1:]):
        assert b <= a + 1e-10, (name, es)
    counts = [r["n_dets"] for r in recs]
    assert counts == sorted(counts), counts
    assert recs[0]["n_dets"] < full.N_dets  # the loosest threshold selects a proper subspace
    assert recs[-1]["n_dets"] == full.N_dets
    assert abs(es[-1] - e_full) < 1e-9, (es[-1], e_full)
    assert all(e >= e_full - 1e-9 for e in es)  # variational


def test_selected_space_matches_oracle_submatrix(case):
    """A middle selection: its sigma and lowest root against the oracle's dense H on the same determinants."""
    from polyquant_gb300.detset import POLYQUANT_DETSET

    name, p, recs, full, e_full = case
    rec = recs[len(recs) // 2]
    prob = _problem(p)
    sel = POLYQUANT_DETSET(prob["n_orb"], prob["n_alpha"], prob["n_beta"], prob["h1"], prob["eri"],
                           restricted=prob["restricted"], charge=prob["charge"], selected_strings=rec["strings"])
    try:
        ns = len(prob["n_orb"])
        # the selected strings come back in the reference layout (last word = orbitals 0..63)
        for s in range(ns):
            for sp in range(2):
                assert list(sel.strings(s, sp)[:, -1]) == rec["strings"][s][sp]
        # determinant (string tuple) -> index in the full space, through the full handle's strings
        fs = [[list(full.strings(s, sp)[:, -1]) for sp in range(2)] for s in range(ns)]
        pos = [[{m: i for i, m in enumerate(fs[s][sp])} for sp in range(2)] for s in range(ns)]
        fidx = {tuple(t): i for i, t in enumerate(full.det_unfold())}
        su = sel.det_unfold()
        idx = np.array([fidx[tuple(pos[k // 2][k % 2][rec["strings"][k // 2][k % 2][t[k]]] for k in range(2 * ns))]
                        for t in su])
        H = O.Detset(p).dense_ham()[np.ix_(idx, idx)]
        C = np.random.default_rng(1).standard_normal((sel.N_dets, 3))
        S = sel.sigma(torch.from_numpy(C).cuda()).cpu().numpy()
        S_ref = H @ C
        assert np.abs(S - S_ref).max() <= 1e-10 * np.abs(S_ref).max(), name
        e, info = sel.davidson(num_states=1, num_subspace_vec=8, convergence_E=1e-10)
        assert abs(e[0] - rec["energies"][0]) < 1e-9
        assert abs(e[0] - np.linalg.eigvalsh(H)[0]) < 1e-9
    finally:
        sel.close()


def test_selected_lists_are_checked():
    import ctypes

    from polyquant_gb300 import _lib
    from polyquant_gb300.detset import make_desc

    p = synthetic_fci(6, 2, 2, seed=1)
    d, keep = make_desc(**{k: v for k, v in batch_dict(p).items() if k != "max_collective_excitation_level"})
    L = _lib.load()
    for bad in ([0b11, 0b101, 0b11], [0b111], [0b11 | (1 << 6)]):  # duplicate, wrong count, orbital 6 of 6
        lists = [np.array(bad, dtype=np.uint64), np.array([0b11], dtype=np.uint64)]
        ptrs = (ctypes.c_void_p * 2)(*[a.ctypes.data for a in lists])
        counts = (ctypes.c_int64 * 2)(*[len(a) for a in lists])
        h = ctypes.c_void_p()
        assert L.pq_ci_create_selected(ctypes.byref(d), ptrs, counts, None, ctypes.byref(h)) == _lib.PQ_ERR_ARG
        assert "pq_ci_create_selected" in _lib.last_error()
