"""Single Hamiltonian elements through the C ABI (pq_ci_element / pq_ci_elements): operator()(i, j) =
Slater_Condon(i, j) (src/ci/determinant_set.hpp:139, src/ci/detset/slater_condon.cpp:4-100) against the oracle's
dense H (its generic Slater_Condon restatement), for one species and electron + positron product spaces, and
unchanged after an explicit matrix was built with a screening threshold that prunes elements
(create_ham + ham.prune, explicit_ham.cpp:51-84)."""
import numpy as np
import pytest

import oracle as O
from cases import batch_dict, h2o_problem, synthetic_ep, synthetic_fci, synthetic_unrestricted

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative to max |H|: elements are exact FP64 from the same formulas

CASES = {
    "h2o_cisd": lambda h2o: h2o_problem(h2o("library"), [2, 2, 2]),
    "fci_8o_4a3b": lambda h2o: synthetic_fci(8, 4, 3, seed=5),
    "unrestricted_7o_3a2b": lambda h2o: synthetic_unrestricted(7, 3, 2, seed=1),
    "ep_cis": lambda h2o: synthetic_ep(6, 2, 1, 5, 1, 0, seed=2, ex_e=[1, 1, 1], ex_p=[1, 1, 1]),
    "ep_coll3_2pos": lambda h2o: synthetic_ep(5, 2, 2, 4, 1, 1, seed=4, max_coll=3),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request, h2o):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    p = CASES[request.param](h2o)
    ref = O.Detset(p)
    g = POLYQUANT_DETSET(**batch_dict(p))
    yield request.param, ref, ref.dense_ham(), g
    g.close()


def _pairs(H, rng, n_pairs=4000):
    """Every connected pair (up to n_pairs of them, sampled), the diagonal, and as many unconnected pairs."""
    n = H.shape[0]
    I, J = np.nonzero(H)
    if len(I) > n_pairs:
        k = rng.choice(len(I), n_pairs, replace=False)
        I, J = I[k], J[k]
    zi = rng.integers(0, n, n_pairs)
    zj = rng.integers(0, n, n_pairs)
    return np.concatenate([I, zi, np.arange(n)]), np.concatenate([J, zj, np.arange(n)])


def test_elements_match_dense_hamiltonian(case):
    name, ref, H, g = case
    rng = np.random.default_rng(0)
    I, J = _pairs(H, rng)
    got = g.elements(I, J)
    scale = np.abs(H).max()
    assert np.abs(got - H[I, J]).max() <= TOL * scale, name
    # the single-pair entry point and the reference-named operator give the same numbers
    for k in rng.choice(len(I), 40, replace=False):
        i, j = int(I[k]), int(J[k])
        assert abs(g(i, j) - H[i, j]) <= TOL * scale
        assert g.Slater_Condon(i, j) == g(i, j)
        assert abs(ref.slater_condon(i, j) - H[i, j]) <= TOL * scale


def test_elements_exact_after_screened_explicit_matrix(case):
    """Elements pruned from the explicit matrix still come back exact (the reference's operator() calls the
    exact Slater_Condon whatever ham.prune removed)."""
    name, ref, H, g = case
    off = np.abs(H[np.triu_indices_from(H, 1)])
    thr = float(np.quantile(off[off > 0], 0.5))  # prunes about half of the nonzero off-diagonal elements
    g.create_ham(screening_threshold=thr, use_for_sigma=True)
    try:
        I, J = np.nonzero((np.abs(H) <= thr) & (H != 0))
        assert len(I) > 0, name
        got = g.elements(I, J)
        assert np.abs(got - H[I, J]).max() <= TOL * np.abs(H).max()
        assert np.all(got != 0.0)
        i, j = int(I[0]), int(J[0])
        assert abs(g(i, j) - H[i, j]) <= TOL * np.abs(H).max()
    finally:
        g.release_ham()


def test_element_index_errors(case):
    from polyquant_gb300._lib import PQError

    _, ref, _, g = case
    n = ref.n_dets
    with pytest.raises(IndexError):
        g(n, 0)
    with pytest.raises(IndexError):
        g(0, -1)
    import ctypes

    from polyquant_gb300 import _lib

    v = ctypes.c_double()
    assert _lib.load().pq_ci_element(g._h, n, 0, ctypes.byref(v)) == _lib.PQ_ERR_ARG
    assert "outside" in _lib.last_error()
    with pytest.raises(PQError):
        _lib.check(_lib.load().pq_ci_element(g._h, -3, 0, ctypes.byref(v)), "pq_ci_element")
