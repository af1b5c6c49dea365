"""<S^2> and the 1-RDM of CI vectors on the GPU (evaluate_s2, src/ci/detset/s2.cpp:4-123; create_1rdm,
src/ci/detset/rdm1.cpp:4-72) against the oracle's restatement of the same routines."""
import numpy as np
import pytest

import oracle as O
from cases import batch_dict, h2o_problem, synthetic_fci

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["h2o_cisd", "fci_6o_3a2b", "fci_7o_3a3b"])
def case(request, h2o):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    p = {"h2o_cisd": lambda: h2o_problem(h2o("library"), [2, 2, 2]),
         "fci_6o_3a2b": lambda: synthetic_fci(6, 3, 2, seed=2),
         "fci_7o_3a3b": lambda: synthetic_fci(7, 3, 3, seed=3)}[request.param]()
    d = O.Detset(p)
    g = POLYQUANT_DETSET(**batch_dict(p))
    w, V = np.linalg.eigh(d.dense_ham())
    yield p, d, g, w, V
    g.close()


def test_s2_matches_restatement_and_is_a_spin_value(case):
    p, d, g, w, V = case
    X = V[:, :4]
    s2 = g.s2(torch.from_numpy(X).cuda())
    ref = d.evaluate_s2(X)[:, 0]
    assert np.abs(s2 - ref).max() < 1e-10
    # eigenvectors of H are spin eigenstates: S(S+1) with S = |n_a - n_b|/2, +1, ...
    S = np.sqrt(s2 + 0.25) - 0.5
    assert np.abs(S - np.round(2 * S) / 2).max() < 1e-6
    rng = np.random.default_rng(1)
    Y = rng.standard_normal((d.n_dets, 9))
    assert np.abs(g.s2(torch.from_numpy(Y).cuda()) - d.evaluate_s2(Y)[:, 0]).max() < 1e-9 * np.abs(Y).max() ** 2 * d.n_dets


def test_rdm1_matches_restatement(case):
    p, d, g, w, V = case
    n = p.n_orb[0]
    c = V[:, 0]
    for spin, ne in ((0, p.n_alpha[0]), (1, p.n_beta[0])):
        R = g.rdm1(torch.from_numpy(c).cuda(), spin)
        ref = d.create_1rdm(c, 0, spin)
        assert np.abs(R - ref).max() < 1e-12
        assert abs(np.trace(R) - ne) < 1e-10
        assert np.abs(R - R.T).max() < 1e-12
        ev = np.linalg.eigvalsh(R)
        assert ev.min() > -1e-10 and ev.max() < 1 + 1e-10


@pytest.mark.parametrize("args", [(5, 2, 2, 4, 1, 1, 3), (6, 2, 1, 5, 1, 0, 4)])
def test_two_species_s2_and_rdm1(args):
    from cases import synthetic_ep
    from polyquant_gb300.detset import POLYQUANT_DETSET

    ne, ea, eb, npo, pa, pb, seed = args
    p = synthetic_ep(ne, ea, eb, npo, pa, pb, seed=seed)
    d = O.Detset(p)
    g = POLYQUANT_DETSET(**batch_dict(p))
    w, V = np.linalg.eigh(d.dense_ham())
    X = V[:, :3]
    s2 = g.s2(torch.from_numpy(X).cuda())
    assert s2.shape == (3, 2)
    for sp in (0, 1):
        assert np.abs(s2[:, sp] - d.evaluate_s2(X)[:, sp]).max() < 1e-10
        S = np.sqrt(s2[:, sp] + 0.25) - 0.5
        assert np.abs(S - np.round(2 * S) / 2).max() < 1e-6
    c = V[:, 0]
    for sp, nelec in ((0, (ea, eb)), (1, (pa, pb))):
        for spin in (0, 1):
            R = g.rdm1(torch.from_numpy(c).cuda(), spin=spin, species=sp)
            assert np.abs(R - d.create_1rdm(c, sp, spin)).max() < 1e-12
            assert abs(np.trace(R) - nelec[spin]) < 1e-10
    g.close()
