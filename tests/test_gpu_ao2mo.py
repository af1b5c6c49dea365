"""AO->MO transform on the GPU (pq_ao2mo) against the numpy restatement of
transform_mo_2_body_integrals (integral.cpp:207-477) and the reference's
pyscf MO-integral fixture (ci_test.cpp:42-70).

Tolerances: FP64 path 1e-11 relative to max|(ij|kl)|; split-precision
tensor-core paths (FP32 accumulation): BF16x3 2e-4, TF32x3 2e-5 relative.
"""
import numpy as np
import pytest

import oracle as O
from polyquant_gb300 import synthetic

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "bf16x3": 2e-4, "tf32x3": 2e-5}


def _modes():
    from polyquant_gb300._lib import PQ_XFORM_BF16X3, PQ_XFORM_FP64, PQ_XFORM_TF32X3

    return {"fp64": PQ_XFORM_FP64, "bf16x3": PQ_XFORM_BF16X3, "tf32x3": PQ_XFORM_TF32X3}


def _packed_case(n, L=64, seed=0, n_mo=None):
    packed = synthetic.ao_eri_packed8(n, seed=seed, L=L)
    C = synthetic.mo_coefficients(n, n_mo, seed=seed + 1)
    full = O.unpack_packed8(packed, n)
    ref = O.ao2mo_full(full, C, C)
    return packed, C, ref


def test_h2o_sto3galls_against_reference_fixture(h2o, golden):
    from polyquant_gb300.integral import ao2mo

    r = h2o("alls")
    C = r["C"]
    n = C.shape[0]
    packed = synthetic.packed8_from_pairs(O.pack_pairs(r["eri"]))
    out = ao2mo(torch.from_numpy(packed).cuda(), torch.from_numpy(C).cuda()).cpu().numpy()
    ref = O.ao2mo_full(r["eri"], C, C)
    assert np.abs(out - ref).max() < 1e-12
    fx = golden["alls_eri"]
    idx = 0
    for i in range(n):
        for j in range(i, n):
            for k in range(n):
                for l in range(k, n):
                    assert abs(abs(out[O.idx2(i, j), O.idx2(k, l)]) - abs(fx[idx, 4])) < 1e-5
                    idx += 1


@pytest.mark.parametrize("mode", ["fp64", "bf16x3", "tf32x3"])
@pytest.mark.parametrize("n,n_mo", [(24, 24), (30, 27), (40, 32), (64, 64), (136, 120)])
def test_packed8_transform(mode, n, n_mo):
    from polyquant_gb300.integral import ao2mo

    packed, C, ref = _packed_case(n, n_mo=n_mo, seed=n)
    out = ao2mo(torch.from_numpy(packed).cuda(), torch.from_numpy(C).cuda(), mode=_modes()[mode]).cpu().numpy()
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < TOL[mode], err


def test_frozen_core_and_deleted_virtuals():
    from polyquant_gb300.integral import transform_mo_2_body_integrals

    n = 20
    packed, C, _ = _packed_case(n, seed=3)
    full = O.unpack_packed8(packed, n)
    Ct = torch.from_numpy(C).cuda()
    out = transform_mo_2_body_integrals(0, 0, Ct, Ct, 5, 5, [2], [3], torch.from_numpy(packed).cuda()).cpu().numpy()
    Cs = C[:, 2:n - 3]
    ref = O.ao2mo_full(full, Cs, Cs)
    assert out.shape == ref.shape
    assert np.abs(out - ref).max() < 1e-11 * np.abs(ref).max()


def test_two_species_pair_matrix():
    """e-p block: (mu nu | la si) with mu nu from species a (10 AOs) and la si from b (7 AOs)."""
    from polyquant_gb300._lib import PQ_AO_PAIRS
    from polyquant_gb300.integral import ao2mo

    na, nb = 10, 7
    rng = np.random.default_rng(4)
    Ba = synthetic._pair_matrix(synthetic._sym_noise(rng, 16, na, 1.0, 4.0))
    Bb = synthetic._pair_matrix(synthetic._sym_noise(rng, 16, nb, 1.0, 4.0))
    P = Ba.T @ Bb  # (npair_a x npair_b)
    Ca = synthetic.mo_coefficients(na, 9, seed=5)
    Cb = synthetic.mo_coefficients(nb, 6, seed=6)
    ia, ja = np.tril_indices(na)
    ib, jb = np.tril_indices(nb)
    full = np.zeros((na, na, nb, nb))
    for p, (i, j) in enumerate(zip(ia, ja)):
        for q, (k, l) in enumerate(zip(ib, jb)):
            full[i, j, k, l] = full[j, i, k, l] = full[i, j, l, k] = full[j, i, l, k] = P[p, q]
    ref = O.ao2mo_full(full, Ca, Cb)
    # column-major (npair_a x npair_b) storage = row-major transpose
    src = torch.from_numpy(np.ascontiguousarray(P.T)).cuda()
    out = ao2mo(src, torch.from_numpy(Ca).cuda(), torch.from_numpy(Cb).cuda(), layout=PQ_AO_PAIRS).cpu().numpy()
    assert np.abs(out - ref).max() < 1e-11 * np.abs(ref).max()


def test_mo_one_body():
    from polyquant_gb300.integral import calculate_mo_1_body_integrals

    rng = np.random.default_rng(7)
    F = rng.standard_normal((12, 12))
    F = F + F.T
    C = synthetic.mo_coefficients(12, 12, seed=8)
    h = calculate_mo_1_body_integrals(torch.from_numpy(F).cuda(), torch.from_numpy(C).cuda(), 1, 2).cpu().numpy()
    Cs = C[:, 1:10]
    assert np.abs(h - Cs.T @ F @ Cs).max() < 1e-12


def test_gemm_wait_timeout_returns_status_and_context_survives():
    """Bounded waits of the tensor-core GEMM: with a one-cycle pipeline budget every CTA gives up at its first
    pending wait, waits (with the default budget) for its own loads and MMAs, frees TMEM and returns; the call
    reports PQ_TIMEOUT and the next call on the same context is correct."""
    from polyquant_gb300._lib import PQ_TIMEOUT, PQError, load
    from polyquant_gb300.integral import ao2mo

    packed, C, ref = _packed_case(64, n_mo=64, seed=5)
    P, Cd = torch.from_numpy(packed).cuda(), torch.from_numpy(C).cuda()
    L = load()
    L.pq_debug_set_wait_budget(1)
    try:
        with pytest.raises(PQError) as e:
            ao2mo(P, Cd, mode=_modes()["bf16x3"])
        assert e.value.status == PQ_TIMEOUT
    finally:
        L.pq_debug_set_wait_budget(0)
    out = ao2mo(P, Cd, mode=_modes()["bf16x3"]).cpu().numpy()
    assert np.abs(out - ref).max() / np.abs(ref).max() < TOL["bf16x3"]


def test_workspace_reused_and_released():
    """The split-precision modes keep their work buffers between calls: a second call on the same inputs gives
    the same numbers (no stale state), a call of another size after it is correct, and after
    pq_ao2mo_release_workspace the next call rebuilds them."""
    from polyquant_gb300 import _lib
    from polyquant_gb300.integral import ao2mo

    L = _lib.load()
    out = {}
    for n in (40, 24, 40):
        packed, C, ref = _packed_case(n, seed=n + 1)
        P, Cd = torch.from_numpy(packed).cuda(), torch.from_numpy(C).cuda()
        a = ao2mo(P, Cd, mode=_modes()["bf16x3"]).cpu().numpy()
        b = ao2mo(P, Cd, mode=_modes()["bf16x3"]).cpu().numpy()
        assert np.array_equal(a, b)
        assert np.abs(a - ref).max() / np.abs(ref).max() < TOL["bf16x3"]
        out.setdefault(n, a)
        assert np.array_equal(out[n], a)
    assert L.pq_ao2mo_release_workspace() == _lib.PQ_OK
    packed, C, ref = _packed_case(40, seed=41)
    a = ao2mo(torch.from_numpy(packed).cuda(), torch.from_numpy(C).cuda(), mode=_modes()["tf32x3"]).cpu().numpy()
    assert np.abs(a - ref).max() / np.abs(ref).max() < TOL["tf32x3"]
    assert L.pq_ao2mo_release_workspace() == _lib.PQ_OK
