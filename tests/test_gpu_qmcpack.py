"""QMCPACK multideterminant payload of a GPU CI solution equals the payload built from the oracle's strings and
unfold table for the same vectors (dump_post_mf_for_qmcpack, src/calculation/calculation.cpp:625-660)."""
import numpy as np
import pytest

import oracle as O
from cases import batch_dict, h2o_problem, synthetic_ep
from polyquant_gb300.qmcpack import multidet_payload, multidet_payload_from_detset

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", ["h2o_cisd", "ep"])
def test_payload_from_gpu_detset(which, h2o):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    p = h2o_problem(h2o("library"), [2, 2, 2]) if which == "h2o_cisd" else synthetic_ep(5, 2, 1, 4, 1, 0, seed=2)
    fc = [1] if which == "h2o_cisd" else [2, 0]
    g = POLYQUANT_DETSET(**batch_dict(p))
    e, vecs, info = g.davidson(num_states=2, num_subspace_vec=6, convergence_E=1e-8, return_vectors=True)
    pl = multidet_payload_from_detset(g, vecs, fc)
    d = O.Detset(p)
    strings = [[np.array([int(w[-1]) for w in d.strings(s, sp)], dtype=np.uint64) for sp in range(2)]
               for s in range(p.n_species)]
    ref = multidet_payload(strings, d.unfold(), vecs.cpu().numpy(), p.n_orb, fc)
    assert set(pl) == set(ref)
    for k in ref:
        assert np.array_equal(pl[k], ref[k]), k
    g.close()
