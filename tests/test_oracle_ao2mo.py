"""The factorized AO->MO row oracle (oracle.ao2mo_rows_factorized, used for the N_AO = 256 parity test where
the full four-index tensor does not fit the host) agrees with the direct four-quarter restatement
(oracle.ao2mo_full, integral.cpp:207-477) on a case small enough for both."""
import numpy as np

import oracle as O
from polyquant_gb300 import synthetic


def test_factorized_rows_equal_four_quarter_transform():
    n, n_mo, L = 12, 9, 20
    Bp = synthetic.ao_eri_pairs(n, seed=4, L=L)
    C = synthetic.mo_coefficients(n, n_mo, seed=5)
    full = O.unpack_packed8(synthetic.packed8_from_pairs(Bp.T @ Bp), n)
    ref = O.ao2mo_full(full, C, C)
    rows = np.array([0, 3, 17, ref.shape[0] - 1])
    got = O.ao2mo_rows_factorized(Bp, C, rows, block=7)
    assert got.shape == (4, ref.shape[1])
    assert np.abs(got - ref[rows]).max() <= 1e-13 * np.abs(ref).max()
