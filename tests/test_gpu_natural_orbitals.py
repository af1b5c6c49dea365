"""Natural spin orbitals from GPU CI vectors and the device 1-RDM (calculate_NOs, src/ci/epci.cpp:200-318),
against the reference's H- golden data (tests/unit_tests/ci/ci_test.cpp:854-871) and the oracle chain."""
import numpy as np
import pytest

import oracle as O
from cases import batch_dict, h_minus, synthetic_ep
from polyquant_gb300.natural_orbitals import calculate_NOs

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_h_minus_from_gpu_davidson():
    from polyquant_gb300.detset import POLYQUANT_DETSET

    r = h_minus()
    ds = POLYQUANT_DETSET(**batch_dict(r["problem"]))
    e, vecs, info = ds.davidson(num_states=5, num_subspace_vec=8, convergence_E=1e-10, return_vectors=True)
    assert info["converged"]
    no = calculate_NOs(ds, vecs, [[r["C"]]], NO_states=[0])
    occ, C = no["occ_nso"][0][0][0], no["C_nso"][0][0][0]
    assert np.abs(occ - r["no_occ"] / 2).max() < 1e-6
    assert np.abs(np.abs(C) - np.abs(r["no_ao"])).max() < 1e-3
    # same density matrix as the oracle's create_1rdm on the GPU vector
    c = vecs[:, 0].cpu().numpy()
    ref = O.Detset(r["problem"]).create_1rdm(c, 0, 0)
    assert np.abs(no["dm1"][0][0][0] - ref).max() < 1e-12
    ds.close()


def test_electron_positron_from_gpu_vectors():
    from polyquant_gb300.detset import POLYQUANT_DETSET

    p = synthetic_ep(6, 2, 1, 5, 1, 0, seed=9)
    ds = POLYQUANT_DETSET(**batch_dict(p))
    e, vecs, info = ds.davidson(num_states=2, num_subspace_vec=6, convergence_E=1e-10, return_vectors=True)
    Ce = np.linalg.qr(np.random.default_rng(0).standard_normal((6, 6)))[0]
    no = calculate_NOs(ds, vecs, [[Ce], [np.eye(5)]], NO_states=[0, 1])
    d = O.Detset(p)
    for k in range(2):
        c = vecs[:, k].cpu().numpy()
        assert len(no["dm1"][k][0]) == 2 and len(no["dm1"][k][1]) == 1
        for sp in (0, 1):
            assert np.abs(no["dm1"][k][sp][0] - d.create_1rdm(c, sp, 0)).max() < 1e-12
        # restricted electrons: the beta matrix is a copy of alpha, as in the reference
        assert np.array_equal(no["dm1"][k][0][1], no["dm1"][k][0][0])
        assert abs(no["occ_nso"][k][0][0].sum() - 2) < 1e-10 and abs(no["occ_nso"][k][1][0].sum() - 1) < 1e-10
    ds.close()
