"""The GPU two-species path on the reference's own electron-positron systems (SCF orbitals and integrals from
the oracle, reproducing the reference's SCF test values): Li- + e+ in Li_basis.g94, where the reference pins the
HF diagonal -7.5257234633357024 (tests/unit_tests/ci/ci_test.cpp:578-599), and PsH, where it pins the natural
spin orbitals (ci_test.cpp:873-892)."""
import numpy as np
import pytest

import oracle as O
from cases import batch_dict, li_wpos, psh_wpos
from polyquant_gb300.natural_orbitals import calculate_NOs

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def li():
    from polyquant_gb300.detset import POLYQUANT_DETSET

    r = li_wpos()
    d = O.Detset(r["problem"])
    g = POLYQUANT_DETSET(**batch_dict(r["problem"]))
    yield r, d, g
    g.close()


def test_li_wpos_diagonal_and_sigma(li):
    r, d, g = li
    diag = g.diagonal().cpu().numpy()
    assert abs(diag[0] - -7.5257234633357024) < 1e-6
    assert np.abs(diag - d.diagonal()).max() < 1e-10
    C = np.random.default_rng(4).standard_normal((d.n_dets, 3))
    S = g.sigma(torch.from_numpy(C).cuda()).cpu().numpy()
    ref = d.sigma(C)
    assert np.abs(S - ref).max() <= 1e-10 * np.abs(ref).max()


def test_li_wpos_davidson_and_explicit_matrix(li):
    r, d, g = li
    H = d.dense_ham()
    w = np.linalg.eigvalsh(H)
    e, info = g.davidson(num_states=3, num_subspace_vec=8, convergence_E=1e-10)
    assert info["converged"] and abs(e[0] - w[0]) < 1e-8
    # higher roots: exact eigenvalues of H (a sector the start block cannot reach may be skipped)
    assert all(np.abs(w - x).min() < 1e-8 for x in e)
    g.create_ham()
    rp, col, val = g.ham_csr(upper=False)
    M = np.zeros_like(H)
    for i in range(d.n_dets):
        M[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    assert np.abs(M - H).max() <= 1e-12 * np.abs(H).max()
    g.release_ham()


def test_psh_natural_spin_orbitals_from_gpu():
    from polyquant_gb300.detset import POLYQUANT_DETSET

    r = psh_wpos()
    g = POLYQUANT_DETSET(**batch_dict(r["problem"]))
    e, vecs, info = g.davidson(num_states=5, num_subspace_vec=8, convergence_E=1e-10, return_vectors=True)
    assert info["converged"]
    no = calculate_NOs(g, vecs, [[r["C"][0]], [r["C"][1]]])
    assert abs(no["occ_nso"][0][0][0].sum() - 1.0) < 1e-8 and abs(no["occ_nso"][0][1][0].sum() - 1.0) < 1e-8
    Ce, Cp = np.abs(no["C_nso"][0][0][0][:, 0]), np.abs(no["C_nso"][0][1][0][:, 0])
    assert np.abs(Ce - [0.300771, 0.345285, 0.43364, 0.0889083, 0.00747211]).max() < 1e-6
    assert abs(Cp[0] - 1.36173) < 1e-5 and abs(Cp[1] - 0.428029) < 1e-6
    g.close()
