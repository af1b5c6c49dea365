"""Problem sizing without a GPU (polyquant_gb300.plan): determinant counts equal the oracle's determinant list
(create_excitation, src/ci/detset/determinant_creation.cpp:148-206) and the Davidson buffers follow the solver's
allocation rule."""
import pytest

import oracle as O
from cases import synthetic_ep, synthetic_fci
from polyquant_gb300.plan import count_determinants, davidson_device_bytes, string_counts


@pytest.mark.parametrize("p", [
    synthetic_fci(7, 3, 2, seed=1),
    synthetic_fci(8, 4, 4, seed=1, ex=[2, 2, 2]),
    synthetic_fci(9, 4, 4, seed=1, ex=[3, 3, 3]),
    synthetic_fci(8, 4, 3, seed=1, ex=[2, 1, 2]),
    synthetic_ep(6, 2, 1, 5, 1, 0, seed=2, ex_e=[1, 1, 1], ex_p=[1, 1, 1]),
    synthetic_ep(5, 2, 2, 4, 1, 1, seed=4, max_coll=3),
    synthetic_ep(6, 3, 3, 6, 1, 1, seed=8, ex_e=[2, 2, 2]),
    synthetic_ep(6, 3, 2, 5, 1, 1, seed=3, ex_e=[2, 2, 3], ex_p=[1, 1, 2], max_coll=2),
], ids=lambda p: f"{p.n_orb}-{p.n_alpha}-{p.n_beta}-{p.ex_level}-{p.max_collective}")
def test_counts_match_the_oracle(p):
    d = O.Detset(p)
    assert count_determinants(p.n_orb, p.n_alpha, p.n_beta, p.ex_level, p.max_collective) == d.n_dets


def test_headline_sizes_and_errors():
    assert count_determinants([16], [8], [8], [[8, 8, 16]]) == 165_636_900
    assert string_counts(16, 8, 8)[1] == 64 and sum(string_counts(16, 8, 8)) == 12_870
    with pytest.raises(ValueError, match="virtual"):
        string_counts(5, 3, 3)
    # one species: the collective limit caps the total level
    assert count_determinants([6], [3], [3], [[2, 2, 4]], 1) == count_determinants([6], [3], [3], [[2, 2, 1]])


def test_davidson_bytes():
    n = 165_636_900
    # 4 roots, 20 start vectors -> m_max = max(40, 40) = 40, T = n x 20
    b = davidson_device_bytes(n, 4, 20)
    assert b == 8 * n * (2 * 40 + 2 * 4 + 20) + 2 * 8 * 4 * (n + 1)
    assert davidson_device_bytes(10, 2, 5, max_subspace=50) == 8 * 10 * (2 * 10 + 4 + 5) + 64 * 11
    # mixed precision on full CI adds the FP32 sigma's two transposed copies; an explicit matrix its CSR
    base = davidson_device_bytes(n, 4, 20)
    assert davidson_device_bytes(n, 4, 20, precision=1) == base + 2 * 16 * (n + 1)
    assert davidson_device_bytes(n, 4, 20, precision=1, full_ci=False) == base
    assert davidson_device_bytes(100, 2, 5, explicit_nnz=1000) == davidson_device_bytes(100, 2, 5) + 12000 + 808


def test_fp32_same_spin_bytes_counts_the_gemm_buffers():
    """The FP32 same-spin GEMM buffers of FCI(16o, 8a8b): one shared dense doubles matrix (12 870 x 12 928,
    FP16 hi and lo), the vector operand (4 x 12 870 rows of 12 928, FP16 hi and lo), two Coulomb tables and
    the scatter-list bound; none when the path does not apply."""
    from polyquant_gb300.plan import davidson_device_bytes, fp32_same_spin_bytes

    n, ldk, npair = 12870, 12928, 136
    want = 2 * 2 * n * ldk + 2 * 2 * 4 * n * ldk + 4 * npair * 2 * n + 16 * n * 64
    assert fp32_same_spin_bytes(16, 8, 8) == want
    # unrestricted integrals: two dense matrices
    assert fp32_same_spin_bytes(16, 8, 8, restricted=False) == want + 2 * 2 * n * ldk
    # too few strings, too many orbitals for the tensor-core path
    assert fp32_same_spin_bytes(10, 5, 4) == 0 and fp32_same_spin_bytes(18, 9, 9) == 0
    base = davidson_device_bytes(165_636_900, 4, 8, precision=1)
    assert davidson_device_bytes(165_636_900, 4, 8, precision=1, same_spin=(16, 8, 8, True)) == base + want
    assert davidson_device_bytes(165_636_900, 4, 8, precision=0, same_spin=(16, 8, 8, True)) == \
        davidson_device_bytes(165_636_900, 4, 8, precision=0)
