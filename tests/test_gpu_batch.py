"""GPU parity of the batched sigma and lockstep Davidson (pq_ci_batch_*).

Each problem of a batch is compared with the oracle's sigma
(sigma_one_species_class_singleshot, direct_singleparticle.cpp:238-372;
sigma_two_species_class_singleshot, direct_mixedparticle.cpp:269-611) and with
the single-problem GPU path, on a batch that mixes electron-only problems,
problems with one and with two positrons, and an unrestricted problem.
"""
import numpy as np
import pytest

import oracle as O
from cases import batch_dict, synthetic_ep, synthetic_fci, synthetic_unrestricted

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SIGMA_RTOL_FP64 = 1e-10
SIGMA_RTOL_FP32 = 2e-5


def mixed_problems():
    return [
        synthetic_fci(6, 3, 2, seed=1),
        synthetic_ep(5, 2, 2, 4, 1, 0, seed=3),  # one positron: 4 positron determinants
        synthetic_ep(6, 2, 2, 4, 1, 1, seed=5),  # two positrons: 16
        synthetic_fci(7, 3, 3, seed=2),
        synthetic_ep(4, 2, 1, 6, 1, 1, seed=7),  # 36 positron determinants
        synthetic_unrestricted(6, 3, 3, seed=4),
        synthetic_ep(6, 3, 3, 6, 1, 0, seed=9),  # 2400 determinants
        synthetic_fci(4, 2, 2, seed=6),
    ]


def reachable_eigs(H, n_start, k, steps=60):
    """Lowest k eigenvalues of H in the block Krylov space of the Davidson start vectors (unit vectors at the
    n_start smallest diagonal elements): with restricted integrals a start space of one spin symmetry never
    reaches states of another, for this solver as for the reference's unit-vector start."""
    dg = np.diag(H)
    idx = np.argsort(dg, kind="stable")[:n_start]
    V = np.zeros((len(dg), n_start))
    V[idx, np.arange(n_start)] = 1.0
    Q = V
    for _ in range(steps):
        Q, _ = np.linalg.qr(np.hstack([Q, H @ Q[:, -n_start:]]))
        if Q.shape[1] >= len(dg):
            break
    return np.linalg.eigvalsh(Q.T @ H @ Q)[:k]


@pytest.fixture(scope="module")
def batch():
    from polyquant_gb300.batch import CIBatch

    probs = mixed_problems()
    refs = [O.Detset(p) for p in probs]
    b = CIBatch([batch_dict(p) for p in probs])
    yield probs, refs, b
    b.close()


def test_sizes(batch):
    probs, refs, b = batch
    assert b.n_dets == [r.n_dets for r in refs]


@pytest.mark.parametrize("nvec", [1, 2, 3, 5])
def test_batch_sigma_fp64(batch, nvec):
    _, refs, b = batch
    rng = np.random.default_rng(nvec)
    Cs = [rng.standard_normal((r.n_dets, nvec)) for r in refs]
    S = b.sigma([torch.from_numpy(C).cuda() for C in Cs])
    for r, C, s in zip(refs, Cs, S):
        S_ref = r.sigma(C)
        assert np.abs(s.cpu().numpy() - S_ref).max() <= SIGMA_RTOL_FP64 * np.abs(S_ref).max()


def test_batch_sigma_fp32(batch):
    from polyquant_gb300._lib import PQ_FP32

    _, refs, b = batch
    rng = np.random.default_rng(11)
    Cs = [rng.standard_normal((r.n_dets, 2)) for r in refs]
    S = b.sigma([torch.from_numpy(C).cuda() for C in Cs], precision=PQ_FP32)
    for r, C, s in zip(refs, Cs, S):
        S_ref = r.sigma(C)
        assert np.abs(s.cpu().numpy() - S_ref).max() <= SIGMA_RTOL_FP32 * np.abs(S_ref).max()


def test_autotuned_shape(batch):
    _, _, b = batch
    t = b.tuning()
    assert t["warps_per_cta"] in (4, 8) and t["rows_per_unit"] >= 1


def test_batch_davidson_fp64(batch):
    _, refs, b = batch
    e, info = b.davidson(num_states=2, num_subspace_vec=4, convergence_E=1e-9)
    for r, ei, inf in zip(refs, e, info):
        H = r.dense_ham()
        assert inf["converged"]
        assert abs(ei[0] - np.linalg.eigvalsh(H)[0]) < 1e-9
        assert np.abs(ei - reachable_eigs(H, 4, 2)).max() < 1e-9


def test_batch_davidson_mixed_within_1ueh(batch):
    from polyquant_gb300._lib import PQ_FP32

    _, refs, b = batch
    e, info = b.davidson(num_states=2, num_subspace_vec=4, convergence_E=1e-6, precision=PQ_FP32)
    for r, ei, inf in zip(refs, e, info):
        assert inf["converged"]
        assert np.abs(ei - reachable_eigs(r.dense_ham(), 4, 2)).max() < 1e-6


def test_batch_davidson_matches_single_problem_davidson(batch):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    probs, _, b = batch
    e, _ = b.davidson(num_states=2, num_subspace_vec=4, convergence_E=1e-9)
    for p, ei in zip(probs, e):
        es, _ = POLYQUANT_DETSET(**batch_dict(p)).davidson(num_states=2, num_subspace_vec=4, convergence_E=1e-9)
        assert np.abs(ei - es).max() < 1e-9


def test_batch_matches_single_problem_path():
    """Medium problems: batched sigma == pq_ci_sigma of each problem's own handle."""
    from polyquant_gb300.batch import CIBatch
    from polyquant_gb300.detset import POLYQUANT_DETSET
    from polyquant_gb300._lib import PQ_FP32

    probs = [synthetic_fci(10, 5, 5, seed=3), synthetic_ep(8, 4, 3, 6, 1, 1, seed=4),
             synthetic_ep(9, 3, 4, 6, 1, 0, seed=5)]
    b = CIBatch([batch_dict(p) for p in probs])
    singles = [POLYQUANT_DETSET(**batch_dict(p)) for p in probs]
    rng = np.random.default_rng(0)
    Cs = [torch.from_numpy(rng.standard_normal((s.N_dets, 2))).cuda() for s in singles]
    for prec, tol in ((0, 1e-12), (PQ_FP32, 1e-5)):
        S = b.sigma(Cs, precision=prec)
        for s, C, Sb in zip(singles, Cs, S):
            ref = s.sigma(C, precision=prec)
            assert (Sb - ref).abs().max().item() <= tol * ref.abs().max().item()
    b.close()


def test_rejects_truncated_space():
    from polyquant_gb300.batch import CIBatch
    from polyquant_gb300._lib import PQError

    with pytest.raises(PQError, match="full product"):
        CIBatch([batch_dict(synthetic_fci(8, 4, 4, seed=1, ex=[2, 2, 2]))])
