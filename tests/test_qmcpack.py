"""QMCPACK multideterminant payload (dump_post_mf_for_qmcpack, src/calculation/calculation.cpp:625-660;
dump_post_mf_to_hdf5_for_QMCPACK, src/io/hdf5_utilities.cpp:399-467; get_det_withfcorbs,
src/ci/detset/determinant_creation.cpp:391-454)."""
import numpy as np
import pytest

import oracle as O
from cases import h2o_problem, synthetic_ep
from polyquant_gb300.qmcpack import multidet_payload, strings_with_frozen_core, write_multidet

M64 = (1 << 64) - 1


def withfc_reference_steps(det_words, nfc, num_int):
    """The reference's word-wise shift: det_words[0] is the highest word; returns words highest first."""
    if nfc == 0:
        return list(det_words) if num_int == len(det_words) else [0] + list(det_words)
    new = []
    if num_int != len(det_words):
        new.append((det_words[0] >> (64 - nfc)) & ((1 << nfc) - 1))
    for c, w in enumerate(det_words):
        j = (w << nfc) & M64
        if c + 1 != len(det_words):
            j |= (det_words[c + 1] >> (64 - nfc)) & ((1 << nfc) - 1)
        if c == len(det_words) - 1:
            j |= (1 << nfc) - 1
        new.append(j)
    return new


@pytest.mark.parametrize("n_orb,nfc", [(10, 0), (10, 1), (20, 5), (40, 30), (63, 1), (50, 14), (33, 63)])
def test_frozen_core_reinsertion_matches_reference_word_shift(n_orb, nfc):
    rng = np.random.default_rng(n_orb * 100 + nfc)
    masks = rng.integers(0, 1 << min(n_orb, 62), size=50, dtype=np.int64).astype(np.uint64)
    n_words = ((n_orb + nfc) >> 6) + 1
    got = strings_with_frozen_core(masks, nfc, n_words)
    for k, m in enumerate(masks):
        ref_high_first = withfc_reference_steps([int(m)], nfc, n_words)
        assert [int(x) for x in got[k]] == ref_high_first[::-1]   # the writer stores words lowest first
        full = (int(m) << nfc) | ((1 << nfc) - 1)
        assert sum(int(x) << (64 * j) for j, x in enumerate(got[k])) == full


def payload_of(d, p, C, fc=None):
    strings = [[np.array([int(w[-1]) for w in d.strings(s, sp)], dtype=np.uint64) for sp in range(2)]
               for s in range(p.n_species)]
    return multidet_payload(strings, d.unfold(), C, p.n_orb, fc)


def test_payload_one_species(h2o, tmp_path):
    p = h2o_problem(h2o("library"), [2, 2, 2])
    d = O.Detset(p)
    C = np.random.default_rng(0).standard_normal((d.n_dets, 2))
    pl = payload_of(d, p, C, [1])
    assert int(pl["NbDet"]) == 141 and int(pl["Nbits"]) == 1 and int(pl["nexcitedstate"]) == 2
    assert int(pl["nstate"]) == 8
    u = d.unfold()
    for sp in range(2):
        masks = [int(w[-1]) for w in d.strings(0, sp)]
        ci = pl[f"CI_{sp}"]
        assert ci.shape == (141, 1) and ci.dtype == np.uint64
        for k in (0, 7, 140):
            assert int(ci[k, 0]) == (masks[u[k, sp]] << 1) | 1
    assert np.array_equal(pl["Coeff"], C[:, 0]) and np.array_equal(pl["Coeff_1"], C[:, 1])
    try:
        import h5py  # noqa: F401
    except ImportError:
        # without h5py the HDF5 writer refuses instead of silently writing another format
        with pytest.raises(RuntimeError, match="h5py"):
            write_multidet(str(tmp_path / "Multidet_h2o.h5"), pl)
    out = write_multidet(str(tmp_path / "Multidet_h2o.h5"), pl, allow_npz=True)
    back = np.load(out) if out.endswith(".npz") else None
    if back is not None:
        assert set(back.files) == set(pl) and np.array_equal(back["CI_1"], pl["CI_1"])


def test_payload_two_species():
    p = synthetic_ep(5, 2, 1, 4, 1, 0, seed=2)
    d = O.Detset(p)
    C = np.random.default_rng(1).standard_normal((d.n_dets, 1))
    pl = payload_of(d, p, C)
    assert sorted(k for k in pl if k.startswith("CI_")) == ["CI_0", "CI_1", "CI_2", "CI_3"]
    u = d.unfold()
    pos = [int(w[-1]) for w in d.strings(1, 0)]
    assert all(int(pl["CI_2"][k, 0]) == pos[u[k, 2]] for k in range(d.n_dets))
    assert np.all(pl["CI_3"] == 0)  # no beta positron
    assert int(pl["nstate"]) == 5


def test_reference_get_det_withfcorbs_cases():
    """tests/unit_tests/ci/ci_test.cpp:148-211: with two frozen orbitals the active HF string 00111 becomes
    0011111; with max_orb = 75 the two-word string {0, 2^63 + 1} (highest word first) becomes {2, 7}."""
    got = strings_with_frozen_core(np.array([0b00111], dtype=np.uint64), 2, 1)
    assert int(got[0, 0]) == 0b0011111
    assert int(strings_with_frozen_core(np.array([0b0011111], dtype=np.uint64), 0, 1)[0, 0]) == 0b0011111
    n_words = ((75 + 2) >> 6) + 1
    got = strings_with_frozen_core(np.array([(1 << 63) + 1], dtype=np.uint64), 2, n_words)
    assert [int(x) for x in got[0][::-1]] == [2, 7]
