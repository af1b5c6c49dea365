"""CPU checks of the batched uneven-CI workload and of the product layout the batched kernel assumes."""
import numpy as np

import oracle as O
from cases import synthetic_ep
from polyquant_gb300 import synthetic


def test_batch_specs_distribution():
    specs = synthetic.batch_specs(256, seed=0)
    assert len(specs) == 256
    for s in specs:
        assert 8 <= s["n_orb"] <= 14
        assert 2 <= s["n_alpha"] <= s["n_orb"] // 2 and 2 <= s["n_beta"] <= s["n_orb"] // 2
        assert s["n_pos"] in (0, 1, 2)
    sizes = np.array([synthetic.batch_spec_dets(s) for s in specs])
    # realised sizes of seed 0 (heavy-tailed)
    assert sizes.sum() == 1_592_197_423
    assert sizes.max() == 371_026_656
    assert np.median(sizes) == 340_200.0
    assert len({s["seed"] for s in specs}) == 256


def test_batch_problem_integrals():
    s = dict(n_orb=8, n_alpha=3, n_beta=2, n_pos=2, n_pos_orb=6, seed=5)
    p = synthetic.batch_problem(s)
    ne, npos = 8 * 9 // 2, 6 * 7 // 2
    assert p["eri"][(0, 0, 0, 0)].shape == (ne, ne)
    assert p["eri"][(1, 0, 1, 0)].shape == (npos, npos)
    assert p["eri"][(0, 0, 1, 0)].shape == (ne, npos)
    assert np.allclose(p["eri"][(0, 0, 0, 0)], p["eri"][(0, 0, 0, 0)].T)
    assert np.linalg.eigvalsh(p["eri"][(0, 0, 0, 0)]).min() > -1e-10
    assert p["n_alpha"] == [3, 1] and p["n_beta"] == [2, 1]
    q = synthetic.batch_problem(dict(s, n_pos=0))
    assert q["n_orb"] == [8] and (0, 0, 1, 0) not in q["eri"]


def test_full_product_layout():
    """Full CI per species orders determinants as ((Ia * Nb + Ib) * P + Jp) with Jp = Iap * Nbp + Ibp
    (create_excitation, determinant_creation.cpp:148-206): the row layout of the batched kernel."""
    p = synthetic_ep(5, 2, 2, 4, 1, 1, seed=3)
    d = O.Detset(p)
    na, nb = len(d.strings(0, 0)), len(d.strings(0, 1))
    pa, pb = len(d.strings(1, 0)), len(d.strings(1, 1))
    u = d.unfold()
    assert u.shape == (na * nb * pa * pb, 4)
    idx = ((u[:, 0].astype(np.int64) * nb + u[:, 1]) * pa + u[:, 2]) * pb + u[:, 3]
    assert np.array_equal(idx, np.arange(len(u)))
