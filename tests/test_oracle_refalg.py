"""The reference-faithful sigma restatement (oracle/ref_restated.cpp: hash-map determinant index, linear
det_idx_unfold, pair-once scatter into per-thread private sigma; direct_singleparticle.cpp:238-372,
direct_mixedparticle.cpp:269-611) agrees with the oracle's sigma, so the CPU timings of both describe the same
product H C."""
import numpy as np
import pytest

import oracle as O
from cases import h2o_problem, psh_wpos, synthetic_ep, synthetic_fci, synthetic_unrestricted


@pytest.mark.parametrize("which", ["h2o_cisd", "fci_6o_3a2b", "unrestricted_6o_3a2b", "cisd_8o_4a4b",
                                   "ep_cis", "ep_coll3_2pos", "psh_wpos"])
def test_reference_restatement_matches_oracle(which, h2o):
    p = {"h2o_cisd": lambda: h2o_problem(h2o("file"), [2, 2, 2]),
         "fci_6o_3a2b": lambda: synthetic_fci(6, 3, 2, seed=2),
         "unrestricted_6o_3a2b": lambda: synthetic_unrestricted(6, 3, 2, seed=5),
         "cisd_8o_4a4b": lambda: synthetic_fci(8, 4, 4, seed=3, ex=[2, 2, 2]),
         "ep_cis": lambda: synthetic_ep(6, 2, 1, 5, 1, 0, seed=2, ex_e=[1, 1, 1], ex_p=[1, 1, 1]),
         "ep_coll3_2pos": lambda: synthetic_ep(5, 2, 2, 4, 1, 1, seed=4, max_coll=3),
         "psh_wpos": lambda: psh_wpos()["problem"]}[which]()
    d, r = O.Detset(p), O.RefAlgDetset(p)
    assert r.n_dets == d.n_dets
    C = np.random.default_rng(3).standard_normal((d.n_dets, 3))
    S, S0 = r.sigma(C), d.sigma(C)
    assert np.abs(S - S0).max() <= 1e-13 * np.abs(S0).max()
    assert np.abs(r.sigma(C, nthreads=1) - S0).max() <= 1e-13 * np.abs(S0).max()
