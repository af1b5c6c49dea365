"""Strings of more than 64 orbitals (two 64-bit words per string) against the oracle, which stores strings in
the reference's multi-word layout (n_words = (max_orb >> 6) + 1, word 0 = highest orbitals;
determinant_creation.cpp:13, 62-68; determinant_operations.cpp:17-110 for holes, particles and phases across
words).

Cases: CISD of 2a2b electrons in 70 orbitals, CIS of an unrestricted 3a2b problem in 68 orbitals, the full
1a1b space of 128 orbitals (the largest orbital count; its Coulomb rows no longer fit shared memory), and two
electron + positron spaces with both species above 64 orbitals (one of them a full product). Each checks the
string words, the diagonal, FP64 and FP32 sigma, single elements, <S^2> and the 1-RDM; the small cases also
check the lowest Davidson root against the dense matrix.

Tolerances: FP64 sigma 1e-10 and FP32 sigma 2e-5 relative to max |sigma|; elements and diagonal 1e-12
relative to max |H|; <S^2> and 1-RDM 1e-10.
"""
import numpy as np
import pytest

import oracle as O
from cases import batch_dict, synthetic_ep, synthetic_fci, synthetic_unrestricted

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = {
    "cisd_70o_2a2b": lambda: synthetic_fci(70, 2, 2, seed=3, ex=[2, 2, 2]),
    "cis_unrestricted_68o_3a2b": lambda: synthetic_unrestricted(68, 3, 2, seed=5, ex=[1, 1, 1]),
    "full_128o_1a1b": lambda: synthetic_fci(128, 1, 1, seed=7, ex=[1, 1, 2]),
    "ep_66o_1a1b_x_70o_1p": lambda: synthetic_ep(66, 1, 1, 70, 1, 0, seed=2, ex_e=[1, 1, 1], ex_p=[1, 0, 1]),
    "ep_full_66o_1a_x_65o_1p": lambda: synthetic_ep(66, 1, 0, 65, 1, 0, seed=4, ex_e=[1, 0, 1], ex_p=[1, 0, 1]),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    p = CASES[request.param]()
    ref = O.Detset(p)
    g = POLYQUANT_DETSET(**batch_dict(p))
    yield request.param, p, ref, g
    g.close()
    torch.cuda.empty_cache()


def test_strings_are_two_words_in_reference_layout(case):
    name, p, ref, g = case
    assert ref.n_words == (max(p.n_orb) >> 6) + 1 >= 2
    for s in range(len(p.n_orb)):
        for sp in range(2):
            got = g.strings(s, sp)
            want = ref.strings(s, sp)
            assert got.shape == want.shape, name
            assert np.array_equal(got, want), (name, s, sp)
    assert g.N_dets == ref.n_dets
    assert np.array_equal(g.det_unfold(), ref.unfold())


def test_diagonal_and_sigma_match_oracle(case):
    from polyquant_gb300._lib import PQ_FP32

    name, p, ref, g = case
    n = ref.n_dets
    D = g.diagonal().cpu().numpy()
    D_ref = ref.diagonal()
    assert np.abs(D - D_ref).max() <= 1e-12 * np.abs(D_ref).max(), name
    C = np.random.default_rng(11).standard_normal((n, 3))
    S_ref = ref.sigma(C)
    X = torch.from_numpy(C).cuda()
    S64 = g.sigma(X).cpu().numpy()
    S32 = g.sigma(X, precision=PQ_FP32).cpu().numpy()
    scale = np.abs(S_ref).max()
    assert np.abs(S64 - S_ref).max() <= 1e-10 * scale, name
    assert np.abs(S32 - S_ref).max() <= 2e-5 * scale, name


def test_elements_match_oracle(case):
    name, p, ref, g = case
    n = ref.n_dets
    rng = np.random.default_rng(5)
    # partners of a few determinants (their sigma columns name every connection) plus random pairs
    I = rng.choice(n, 24, replace=False)
    E = np.zeros((n, len(I)))
    E[I, np.arange(len(I))] = 1.0
    H_cols = ref.sigma(E)  # column c = H[:, I[c]]
    cols = []
    for c, i in enumerate(I):
        J = np.nonzero(H_cols[:, c])[0]
        cols.append((np.full(len(J), i), J, H_cols[J, c]))
    Ii = np.concatenate([c[0] for c in cols])
    Jj = np.concatenate([c[1] for c in cols])
    want = np.concatenate([c[2] for c in cols])
    got = g.elements(Ii, Jj)
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= 1e-12 * scale, name
    ri, rj = rng.integers(0, n, 200), rng.integers(0, n, 200)
    want_r = np.array([ref.slater_condon(int(a), int(b)) for a, b in zip(ri, rj)])
    assert np.abs(g.elements(ri, rj) - want_r).max() <= 1e-12 * scale


def test_s2_and_rdm1_match_oracle(case):
    name, p, ref, g = case
    n = ref.n_dets
    C = np.random.default_rng(3).standard_normal((n, 2))
    C /= np.linalg.norm(C, axis=0)
    X = torch.from_numpy(C).cuda()
    s2 = np.asarray(g.evaluate_s2(X))
    s2_ref = np.asarray(ref.evaluate_s2(C)).reshape(s2.shape)
    assert np.abs(s2 - s2_ref).max() <= 1e-10 * max(1.0, np.abs(s2_ref).max()), name
    for s in range(len(p.n_orb)):
        for sp in range(2):
            if (p.n_alpha, p.n_beta)[sp][s] == 0:
                continue
            R = g.rdm1(X[:, 0], spin=sp, species=s)
            R_ref = ref.create_1rdm(C[:, 0], species=s, spin=sp)
            assert np.abs(R - R_ref).max() <= 1e-10, (name, s, sp)


def test_lowest_root_matches_dense(case):
    name, p, ref, g = case
    if ref.n_dets > 5000:
        pytest.skip("dense eigensolve only for the small spaces")
    e, info = g.davidson(num_states=1, convergence_E=1e-10)
    assert info["converged"], name
    w = np.linalg.eigvalsh(ref.dense_ham())
    assert abs(e[0] - w[0]) <= 1e-8 * max(1.0, abs(w[0])), name


def test_explicit_matrix_sigma_matches_oracle(case):
    name, p, ref, g = case
    if ref.n_dets > 40000:
        pytest.skip("explicit matrix only for the smaller spaces")
    g.create_ham(use_for_sigma=True)
    try:
        C = np.random.default_rng(9).standard_normal((ref.n_dets, 2))
        S = g.sigma(torch.from_numpy(C).cuda()).cpu().numpy()
        S_ref = ref.sigma(C)
        assert np.abs(S - S_ref).max() <= 1e-10 * np.abs(S_ref).max(), name
    finally:
        g.release_ham()


def test_orbital_limit_and_batch_refusal():
    import ctypes

    from polyquant_gb300 import _lib
    from polyquant_gb300._lib import PQError
    from polyquant_gb300.batch import CIBatch

    # 129 orbitals are refused before any integral is read (the descriptor carries no integral pointers)
    d = _lib.PQDesc()
    d.n_species = 1
    d.n_orb[0], d.n_alpha[0], d.n_beta[0], d.restricted[0] = 129, 1, 1, 1
    h = ctypes.c_void_p()
    assert _lib.load().pq_ci_create(ctypes.byref(d), None, ctypes.byref(h)) == _lib.PQ_ERR_ARG
    assert "outside 1..128" in _lib.last_error()
    p = synthetic_fci(66, 1, 1, seed=1, ex=[1, 1, 2])
    with pytest.raises(PQError, match="at most 64 orbitals"):
        CIBatch([batch_dict(p)])
