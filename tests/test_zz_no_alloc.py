"""The allocation-free sigma entry point (pq_ci_sigma_noalloc) against pq_ci_sigma.

pq_ci_sigma_noalloc serves callers that may not allocate device memory while
they compute (a pre-reserved memory pool, a loop that must not hit the
synchronisation of cudaMalloc/cudaFree, a solver recorded into a CUDA graph):
its work vectors live in a fixed 2 x 16 MiB array inside the library.  This
file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import pytest

from cases import synthetic_fci

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SIGMA_RTOL_FP64 = 1e-10  # same bar as the other FP64 sigma tests
SIGMA_RTOL_FP32 = 2e-5


def _detset(p):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    return POLYQUANT_DETSET(p.n_orb, p.n_alpha, p.n_beta, p.h1, p.eri, p.ex_level, restricted=p.restricted,
                            charge=p.charge)


def _run(L, fn, g, C, prec):
    n, k = g.N_dets, C.shape[0]
    S = torch.empty_like(C)
    torch.cuda.synchronize()
    st = fn(g._h, ctypes.c_void_p(C.data_ptr()), n, k, ctypes.c_void_p(S.data_ptr()), n, prec)
    torch.cuda.synchronize()
    return st, S


def _scratch_bytes(L, g):
    b = ctypes.c_int64(-1)
    assert L.pq_debug_scratch_bytes(g._h, ctypes.byref(b)) == 0
    return b.value


@pytest.mark.parametrize("prec_name", ["fp64", "fp32"])
def test_noalloc_on_a_fresh_handle_grows_no_handle_memory(prec_name):
    """The entry point's promise: on a handle that never ran pq_ci_sigma, calls leave the handle's
    grow-on-demand work buffers (interleaved vectors, transposed FP32 copies) at zero bytes; the results
    still agree with pq_ci_sigma, which is run afterwards and does grow them."""
    from polyquant_gb300 import _lib

    L = _lib.load()
    prec, rtol = (_lib.PQ_FP64, SIGMA_RTOL_FP64) if prec_name == "fp64" else (_lib.PQ_FP32, SIGMA_RTOL_FP32)
    # full CI, so that FP32 pq_ci_sigma would take the transposing path with its extra buffers
    g = _detset(synthetic_fci(9, 4, 4, seed=45))
    assert _scratch_bytes(L, g) == 0
    gen = torch.Generator(device="cuda").manual_seed(11)
    outs = []
    for k in (4, 2, 4):
        C = torch.randn(k, g.N_dets, device="cuda", dtype=torch.float64, generator=gen)
        st, S = _run(L, L.pq_ci_sigma_noalloc, g, C, prec)
        assert st == _lib.PQ_OK, _lib.last_error()
        assert _scratch_bytes(L, g) == 0
        outs.append((C, S))
    for C, S in outs:
        st_ref, S_ref = _run(L, L.pq_ci_sigma, g, C, prec)
        assert st_ref == _lib.PQ_OK
        assert (S - S_ref).abs().max().item() <= rtol * S_ref.abs().max().item()
    assert _scratch_bytes(L, g) > 0
    g.close()


def test_noalloc_matches_pq_ci_sigma_on_consecutive_calls():
    from polyquant_gb300 import _lib

    L = _lib.load()
    g = _detset(synthetic_fci(8, 4, 4, seed=41))
    n = g.N_dets
    gen = torch.Generator(device="cuda").manual_seed(9)
    # column-major (n x k) == row-major (k x n)
    for k, prec, rtol in ((3, _lib.PQ_FP64, SIGMA_RTOL_FP64), (5, _lib.PQ_FP64, SIGMA_RTOL_FP64),
                          (4, _lib.PQ_FP32, SIGMA_RTOL_FP32), (1, _lib.PQ_FP64, SIGMA_RTOL_FP64)):
        C = torch.randn(k, n, device="cuda", dtype=torch.float64, generator=gen)
        st_ref, S_ref = _run(L, L.pq_ci_sigma, g, C, prec)
        assert st_ref == _lib.PQ_OK, _lib.last_error()
        st, S = _run(L, L.pq_ci_sigma_noalloc, g, C, prec)
        assert st == _lib.PQ_OK, _lib.last_error()
        scale = S_ref.abs().max().item()
        assert (S - S_ref).abs().max().item() <= rtol * scale


def test_noalloc_second_problem_after_first():
    """The shared array keeps the previous call's contents; a different problem must not see them."""
    from polyquant_gb300 import _lib

    L = _lib.load()
    g1 = _detset(synthetic_fci(9, 4, 4, seed=42))
    g2 = _detset(synthetic_fci(7, 3, 3, seed=43))
    for g in (g1, g2, g1):
        C = torch.randn(4, g.N_dets, device="cuda", dtype=torch.float64)
        st_ref, S_ref = _run(L, L.pq_ci_sigma, g, C, _lib.PQ_FP64)
        st, S = _run(L, L.pq_ci_sigma_noalloc, g, C, _lib.PQ_FP64)
        assert st_ref == st == _lib.PQ_OK
        assert (S - S_ref).abs().max().item() <= SIGMA_RTOL_FP64 * S_ref.abs().max().item()


def test_noalloc_rejects_problems_beyond_its_scratch():
    from polyquant_gb300 import _lib

    L = _lib.load()
    g = _detset(synthetic_fci(12, 6, 6, seed=44))  # 853,776 dets x 4 x 8 B > 16 MiB
    C = torch.randn(4, g.N_dets, device="cuda", dtype=torch.float64)
    st, _ = _run(L, L.pq_ci_sigma_noalloc, g, C, _lib.PQ_FP64)
    assert st == _lib.PQ_ERR_ARG
    assert "16 MiB" in _lib.last_error()
    # the same problem still fits one vector at a time in FP32
    C1 = torch.randn(1, g.N_dets, device="cuda", dtype=torch.float64)
    st_ref, S_ref = _run(L, L.pq_ci_sigma, g, C1, _lib.PQ_FP32)
    st, S = _run(L, L.pq_ci_sigma_noalloc, g, C1, _lib.PQ_FP32)
    assert st_ref == st == _lib.PQ_OK
    assert (S - S_ref).abs().max().item() <= SIGMA_RTOL_FP32 * S_ref.abs().max().item()
