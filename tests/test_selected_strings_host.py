"""pq_ci_create_selected (the selected-string extension) rejects malformed string lists before it touches a
device: duplicates, wrong particle counts, orbitals outside the species, empty lists and more than 64
orbitals; the message names the entry point."""
import ctypes

import numpy as np
import pytest

from cases import batch_dict, synthetic_fci
from polyquant_gb300 import _lib
from polyquant_gb300.detset import make_desc


def _call(d, lists):
    arrs = [np.ascontiguousarray(np.asarray(a, dtype=np.uint64)) for a in lists]
    ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data if len(a) else None for a in arrs])
    counts = (ctypes.c_int64 * len(arrs))(*[len(a) for a in arrs])
    h = ctypes.c_void_p()
    return _lib.load().pq_ci_create_selected(ctypes.byref(d), ptrs, counts, None, ctypes.byref(h))


@pytest.mark.parametrize("alpha, why", [
    ([0b11, 0b101, 0b11], "twice"),          # duplicate
    ([0b111], "is not 2 of 6"),              # three electrons in a 2-electron list
    ([0b11 | (1 << 6)], "is not 2 of 6"),    # orbital 6 of 6
    ([], "strings"),                          # empty list
])
def test_malformed_lists_are_rejected(alpha, why):
    p = synthetic_fci(6, 2, 2, seed=1)
    d, keep = make_desc(**batch_dict(p))
    assert _call(d, [alpha, [0b11]]) == _lib.PQ_ERR_ARG
    msg = _lib.last_error()
    assert "pq_ci_create_selected" in msg and why in msg, msg


def test_more_than_64_orbitals_is_rejected():
    d = _lib.PQDesc()
    d.n_species = 1
    d.n_orb[0], d.n_alpha[0], d.n_beta[0], d.restricted[0] = 65, 1, 1, 1
    assert _call(d, [[1], [1]]) == _lib.PQ_ERR_ARG
    assert "outside 1..64" in _lib.last_error()
