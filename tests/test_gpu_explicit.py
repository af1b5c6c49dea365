"""Explicit sparse Hamiltonian (create_ham, src/ci/detset/explicit_ham.cpp:51-84; one species
explicit_ham_singleparticle.cpp, electron + positron explicit_ham_mixedparticle.cpp) against the oracle's dense H."""
import numpy as np
import pytest

import oracle as O
from cases import batch_dict, h2o_problem, synthetic_ep, synthetic_fci, synthetic_unrestricted

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = {
    "h2o_cisd": lambda h2o: h2o_problem(h2o("library"), [2, 2, 2]),
    "h2o_fci": lambda h2o: h2o_problem(h2o("library"), [2, 2, 4]),
    "fci_8o_4a3b": lambda h2o: synthetic_fci(8, 4, 3, seed=5),
    "unrestricted_7o_3a2b": lambda h2o: synthetic_unrestricted(7, 3, 2, seed=1),
    # electron + positron: CIS x CIS, and the full product under a collective excitation limit
    "ep_cis": lambda h2o: synthetic_ep(6, 2, 1, 5, 1, 0, seed=2, ex_e=[1, 1, 1], ex_p=[1, 1, 1]),
    "ep_coll3_2pos": lambda h2o: synthetic_ep(5, 2, 2, 4, 1, 1, seed=4, max_coll=3),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request, h2o):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    p = CASES[request.param](h2o)
    ref = O.Detset(p)
    g = POLYQUANT_DETSET(**batch_dict(p))
    yield request.param, p, ref, g
    g.close()


def dense_from_csr(n, rp, col, val):
    H = np.zeros((n, n))
    for i in range(n):
        H[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    return H


def test_upper_triangle_matches_dense(case):
    _, p, ref, g = case
    H = ref.dense_ham()
    g.create_ham()
    rp, col, val = g.ham_csr(upper=True)
    n = ref.n_dets
    assert np.all(np.diff(rp) >= 1)
    for i in range(n):  # columns ascending, upper triangle, diagonal first
        c = col[rp[i]:rp[i + 1]]
        assert c[0] == i and np.all(np.diff(c) > 0)
    U = dense_from_csr(n, rp, col, val)
    assert np.abs(U - np.triu(H)).max() <= 1e-12 * np.abs(H).max()
    # exact zeros are not stored off the diagonal
    nz = np.count_nonzero(np.triu(H, 1))
    assert len(col) - n == nz
    rpf, colf, valf = g.ham_csr(upper=False)
    assert np.abs(dense_from_csr(n, rpf, colf, valf) - H).max() <= 1e-12 * np.abs(H).max()
    g.release_ham()


def test_screening_threshold(case):
    _, p, ref, g = case
    H = ref.dense_ham()
    thr = 1e-3
    g.create_ham(screening_threshold=thr)
    rp, col, val = g.ham_csr(upper=True)
    U = dense_from_csr(ref.n_dets, rp, col, val)
    expect = np.where(np.abs(np.triu(H)) > thr, np.triu(H), 0.0)
    assert np.abs(U - expect).max() <= 1e-12 * np.abs(H).max()
    assert np.all(np.abs(val) > thr)
    g.release_ham()


def test_sigma_and_davidson_with_explicit_matrix(case):
    _, p, ref, g = case
    C = np.random.default_rng(2).standard_normal((ref.n_dets, 3))
    Cd = torch.from_numpy(C).cuda()
    S_direct = g.sigma(Cd).cpu().numpy()
    g.create_ham(use_for_sigma=True)
    S = g.sigma(Cd).cpu().numpy()
    assert np.abs(S - S_direct).max() <= 1e-12 * np.abs(S_direct).max()
    assert np.abs(S - ref.sigma(C)).max() <= 1e-10 * np.abs(S).max()
    k = 2
    e, info = g.davidson(num_states=k, num_subspace_vec=4, convergence_E=1e-9)
    w = np.linalg.eigvalsh(ref.dense_ham())
    assert info["converged"]
    assert np.abs(e - w[:k]).max() < 1e-9
    g.release_ham()
