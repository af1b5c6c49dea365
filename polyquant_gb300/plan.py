"""Sizing a CI problem before it is built: determinant counts and the device
memory of the Davidson solver, from the problem definition alone (no GPU).

``count_determinants`` counts the determinant list that create_excitation
(src/ci/detset/determinant_creation.cpp:148-206) produces: per species and
spin the strings with k replacements relative to the HF string number
C(n_e, k) * C(n_orb - n_e, k) for k = 0..ex_max (the reference aborts when
ex_max exceeds the virtual orbitals, determinant_creation.cpp:54-56, and so
does this count); a species' (alpha, beta) pair is kept when its total level
is within the species' total limit, and the levels of all species together
within max_collective_excitation_level.  (With one species the product
space is limited by min(total, collective).)

``davidson_device_bytes`` is the device memory the Davidson solver of this
library allocates for a problem of n_dets determinants: the subspace V and
its sigma W (n_dets x m_max each), the Ritz vectors, residuals and a work
block (n_dets x k, n_dets x k, n_dets x max(k, m0)), all FP64, plus the two
interleaved sigma work vectors (4 per determinant, FP64); m_max follows the
reference's choice max(2 * num_subspace_vec, 10 * num_states)
(src/ci/epci.cpp:589-590) unless max_subspace is given.  With
``precision=PQ_FP32`` (mixed) on a one-species full-CI space the FP32 sigma
adds its two transposed vector copies (4 FP32 values per determinant each);
with ``explicit_nnz`` (an explicit matrix built for sigma) the CSR arrays
(12 B per stored entry plus 8 B per row) are counted too, and with
``same_spin`` = (n_orb, n_alpha, n_beta, restricted) the buffers of the FP32
same-spin tensor-core GEMMs (``fp32_same_spin_bytes``).  Handle tables, the
diagonal (8 B per determinant) and the caller's own vectors come on top.

``fp32_same_spin_bytes`` is what the FP32 full-CI sigma of a one-species space
allocates on its first call when its same-spin doubles run as dense GEMMs
(ci_sigma32_ss.cu, the same applicability test): the FP16 hi/lo copies of the
dense doubles matrix of each spin list (shared by both spins when the lists
and integrals coincide), the FP16 hi/lo vector operand, the two Coulomb tables
of the singles and a bound on the alpha-beta kernel's scatter lists.
"""
from __future__ import annotations

from math import comb
from typing import List, Sequence

INT_MAX = 2 ** 31 - 1


def string_counts(n_orb: int, n_e: int, ex_max: int) -> List[int]:
    """Number of strings with exactly k replacements, k = 0..ex_max (reference order groups them by k)."""
    n_virt = n_orb - n_e
    out = []
    for k in range(ex_max + 1):
        if k > n_virt:
            raise ValueError(f"excitation level {k} exceeds the {n_virt} virtual orbitals")
        out.append(comb(n_e, k) * comb(n_virt, k))
    return out


def _pair_levels(n_orb: int, n_alpha: int, n_beta: int, ex: Sequence[int]) -> List[int]:
    """count[L] of kept (alpha, beta) string pairs with total level L <= ex[2]."""
    a = string_counts(n_orb, n_alpha, ex[0])
    b = string_counts(n_orb, n_beta, ex[1])
    out = [0] * (ex[2] + 1)
    for ka, na in enumerate(a):
        for kb, nb in enumerate(b):
            if ka + kb <= ex[2]:
                out[ka + kb] += na * nb
    return out


def count_determinants(n_orb: Sequence[int], n_alpha: Sequence[int], n_beta: Sequence[int],
                       excitation_level: Sequence[Sequence[int]],
                       max_collective_excitation_level: int = INT_MAX) -> int:
    """Length of the determinant list of a one- or two-species problem."""
    ns = len(n_orb)
    if ns not in (1, 2):
        raise ValueError("one or two species")
    mc = max_collective_excitation_level
    if ns == 1:
        ex = list(excitation_level[0])
        ex[2] = min(ex[2], mc)
        return sum(_pair_levels(n_orb[0], n_alpha[0], n_beta[0], ex)) if ex[2] >= 0 else 0
    p0 = _pair_levels(n_orb[0], n_alpha[0], n_beta[0], excitation_level[0])
    p1 = _pair_levels(n_orb[1], n_alpha[1], n_beta[1], excitation_level[1])
    return sum(c0 * c1 for l0, c0 in enumerate(p0) for l1, c1 in enumerate(p1) if l0 + l1 <= mc)


def fp32_same_spin_bytes(n_orb: int, n_alpha: int, n_beta: int, restricted: bool = True) -> int:
    """Device bytes of the FP32 same-spin GEMM path of a one-species full-CI space (0 when it does not apply:
    more than 16 orbitals or 64 alpha singles per string for the tensor-core path, fewer than 256 or more than
    32768 strings of a spin, or doubles filling less than 3 % of a row)."""
    na_s, nb_s = comb(n_orb, n_alpha), comb(n_orb, n_beta)
    singles_a = n_alpha * (n_orb - n_alpha)
    if n_orb > 16 or singles_a > 64 or nb_s >= 32768 or na_s >= 65536:
        return 0
    sides = []
    for n_s, ne in ((na_s, n_alpha), (nb_s, n_beta)):
        doubles = comb(ne, 2) * comb(n_orb - ne, 2)
        if n_s < 256 or n_s > 32768 or doubles < 0.03 * n_s:
            return 0
        sides.append((n_s, (n_s + 63) // 64 * 64))
    shared = restricted and n_alpha == n_beta
    dense = sum(2 * 2 * n_s * ldk for n_s, ldk in (sides[:1] if shared else sides))
    (na_, ldk_a), (nb_, ldk_b) = sides
    operand = 2 * 2 * max(4 * nb_ * ldk_a, 4 * na_ * ldk_b)
    npair = n_orb * (n_orb + 1) // 2
    coulomb = 4 * npair * (na_ + nb_)
    scatter_lists = 16 * nb_ * n_beta * (n_orb - n_beta)
    return dense + operand + coulomb + scatter_lists


def davidson_device_bytes(n_dets: int, num_states: int, num_subspace_vec: int = 5, max_subspace: int = 0,
                          precision: int = 0, full_ci: bool = True, explicit_nnz: int = 0,
                          same_spin: Sequence = None) -> int:
    """Device bytes of the Davidson work arrays for n_dets determinants (see the module docstring).
    precision: 0 = FP64, 1 = mixed (FP32 sigma with FP64 refinement); full_ci: one-species space with every
    (alpha, beta) pair (the FP32 sigma then keeps transposed copies); explicit_nnz: stored entries of an
    explicit matrix that sigma multiplies with (0: none); same_spin: (n_orb, n_alpha, n_beta, restricted) of
    that space, to count the FP32 same-spin GEMM buffers."""
    k = num_states
    m0 = min(max(num_subspace_vec, k), n_dets)
    m_max = max_subspace if max_subspace > 0 else max(2 * num_subspace_vec, 10 * k)
    m_max = min(max(m_max, m0 + k), n_dets)
    vectors = 8 * n_dets * (2 * m_max + 2 * k + max(k, m0))
    sigma_work = 2 * 8 * 4 * (n_dets + 1)
    fp32_transposed = 2 * 4 * 4 * (n_dets + 1) if precision == 1 and full_ci else 0
    csr = (12 * explicit_nnz + 8 * (n_dets + 1)) if explicit_nnz > 0 else 0
    ss = fp32_same_spin_bytes(*same_spin) if (precision == 1 and full_ci and same_spin is not None) else 0
    return vectors + sigma_work + fp32_transposed + csr + ss
