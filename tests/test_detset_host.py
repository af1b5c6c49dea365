"""Host-side argument mapping of the POLYQUANT_DETSET mirror, checked without a GPU by standing in for the
device calls: the reference-named property methods (evaluate_s2, s2.cpp:4-123; create_1rdm, rdm1.cpp:4-72)
forward to the device wrappers with the reference's argument meaning."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def fake_detset(n_species):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    ds = POLYQUANT_DETSET.__new__(POLYQUANT_DETSET)  # no device handle
    ds.n_species = n_species
    ds.N_dets = 6
    ds._h = None
    calls = []

    def s2(C):
        k = C.reshape(6, -1).shape[1]
        out = np.arange(k * n_species, dtype=float).reshape(k, n_species)
        return out[:, 0] if n_species == 1 else out

    def rdm1(c, spin=0, species=0):
        calls.append((c.clone(), spin, species))
        return np.eye(2)

    ds.s2, ds.rdm1 = s2, rdm1
    return ds, calls


@pytest.mark.parametrize("n_species", [1, 2])
def test_evaluate_s2_is_states_by_species(n_species):
    ds, _ = fake_detset(n_species)
    S = ds.evaluate_s2(torch.zeros(6, 3, dtype=torch.float64))
    assert S.shape == (3, n_species)
    assert np.array_equal(S, np.arange(3 * n_species, dtype=float).reshape(3, n_species))


def test_create_1rdm_argument_order():
    ds, calls = fake_detset(2)
    C = torch.arange(18, dtype=torch.float64).reshape(6, 3)
    ds.create_1rdm(2, 1, 0, C)          # state 2, species 1, spin 0
    c, spin, species = calls[-1]
    assert torch.equal(c, C[:, 2]) and spin == 0 and species == 1
    ds.create_1rdm(0, 0, 1, C[:, 1])    # a single vector
    c, spin, species = calls[-1]
    assert torch.equal(c, C[:, 1]) and spin == 1 and species == 0


def test_element_access_checks_indices_before_the_library():
    """operator()(i, j) = Slater_Condon(i, j) (determinant_set.hpp:139) takes determinant indices
    0..N_dets-1: a negative or too large index, or a non-integer, raises before any library call."""
    from polyquant_gb300.detset import POLYQUANT_DETSET

    ds = POLYQUANT_DETSET.__new__(POLYQUANT_DETSET)
    ds._h, ds.N_dets = None, 6
    for i, j in ((-1, 0), (0, -1), (6, 0), (0, 6), (2 ** 40, 1)):
        with pytest.raises(IndexError):
            ds(i, j)
        with pytest.raises(IndexError):
            ds.Slater_Condon(i, j)
    with pytest.raises(TypeError):
        ds(1.0, 2)
    with pytest.raises(IndexError):
        ds.elements([0, 1, 6], [0, 1, 2])
    with pytest.raises(ValueError):
        ds.elements([0, 1], [0])


def test_unfold_and_get_det_mirrors():
    from polyquant_gb300.detset import POLYQUANT_DETSET

    ds = POLYQUANT_DETSET.__new__(POLYQUANT_DETSET)
    ds._h, ds.N_dets, ds.n_species = None, 3, 1
    ds.det_unfold = lambda: np.array([[0, 0], [0, 1], [1, 0]], dtype=np.int32)
    ds.strings = lambda s, sp: np.array([[0b0011], [0b0101]], dtype=np.uint64)
    assert ds.det_idx_unfold(2) == [1, 0]
    with pytest.raises(IndexError):
        ds.det_idx_unfold(3)
    assert int(ds.get_det(0, 1, 1)[0]) == 0b0101
