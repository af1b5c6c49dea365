"""GPU parity of the sigma path (through the C ABI) against the CPU oracle.

Bars: strings, determinant order and excitation structure bit-exact; FP64
diagonal and sigma within 1e-10 relative to max|sigma| (energies within
1e-9 Eh); FP32 sigma within 2e-5 relative.
"""
import numpy as np
import pytest

import oracle as O
from cases import h2o_problem, synthetic_fci, synthetic_unrestricted

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SIGMA_RTOL_FP64 = 1e-10
SIGMA_RTOL_FP32 = 2e-5
ENERGY_TOL = 1e-9


def gpu_detset(p):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    return POLYQUANT_DETSET(p.n_orb, p.n_alpha, p.n_beta, p.h1, p.eri, p.ex_level, restricted=p.restricted,
                            charge=p.charge, max_collective_excitation_level=p.max_collective)


def _cases(h2o):
    out = {
        "h2o_cis": h2o_problem(h2o("file"), [1, 1, 1]),
        "h2o_cisd": h2o_problem(h2o("library"), [2, 2, 2]),
        "h2o_fci": h2o_problem(h2o("library"), [2, 2, 4]),
        "fci_8o_4a3b": synthetic_fci(8, 4, 3, seed=11),
        "cisd_10o_5a5b": synthetic_fci(10, 5, 5, seed=12, ex=[2, 2, 2]),
        "cisdt_9o_4a4b": synthetic_fci(9, 4, 4, seed=13, ex=[3, 3, 3]),
        "unrestricted_7o_3a2b": synthetic_unrestricted(7, 3, 2, seed=14),
        "one_electron_6o": synthetic_fci(6, 1, 0, seed=15),
        # 595 orbital pairs and 93 singles per string: generic (unpacked) path, ERIs read from global
        "cisd_34o_3a3b": synthetic_fci(34, 3, 3, seed=16, ex=[2, 2, 2]),
    }
    return out


CASES = ["h2o_cis", "h2o_cisd", "h2o_fci", "fci_8o_4a3b", "cisd_10o_5a5b", "cisdt_9o_4a4b",
         "unrestricted_7o_3a2b", "one_electron_6o", "cisd_34o_3a3b"]


@pytest.fixture(scope="module")
def cases(h2o):
    return _cases(h2o)


@pytest.mark.parametrize("name", CASES)
def test_strings_and_dets_bit_exact(cases, name):
    p = cases[name]
    ref = O.Detset(p)
    g = gpu_detset(p)
    assert g.N_dets == ref.n_dets
    for sp in range(2):
        assert np.array_equal(g.strings(0, sp), ref.strings(0, sp))
    assert np.array_equal(g.det_unfold(), ref.unfold())


@pytest.mark.parametrize("name", CASES)
def test_diagonal(cases, name):
    p = cases[name]
    ref = O.Detset(p).diagonal()
    d = gpu_detset(p).diagonal().cpu().numpy()
    assert np.abs(d - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("nvec", [1, 2, 3, 5])
def test_sigma_fp64_vs_oracle(cases, name, nvec):
    p = cases[name]
    ref = O.Detset(p)
    g = gpu_detset(p)
    rng = np.random.default_rng(nvec)
    C = rng.standard_normal((ref.n_dets, nvec))
    S_ref = ref.sigma(C)
    S = g.sigma(torch.from_numpy(C).cuda()).cpu().numpy()
    scale = np.abs(S_ref).max()
    assert np.abs(S - S_ref).max() <= SIGMA_RTOL_FP64 * scale
    # host-buffer entry point gives the same result
    S_host = g.sigma(C)
    assert np.abs(S_host - S_ref).max() <= SIGMA_RTOL_FP64 * scale


@pytest.mark.parametrize("name", CASES)
def test_sigma_fp32_vs_oracle(cases, name):
    from polyquant_gb300._lib import PQ_FP32

    p = cases[name]
    ref = O.Detset(p)
    g = gpu_detset(p)
    C = np.random.default_rng(7).standard_normal((ref.n_dets, 4))
    S_ref = ref.sigma(C)
    S = g.sigma(torch.from_numpy(C).cuda(), precision=PQ_FP32).cpu().numpy()
    assert np.abs(S - S_ref).max() <= SIGMA_RTOL_FP32 * np.abs(S_ref).max()


def test_sigma_reference_patterns_h2o(cases):
    """The reference's fast-vs-slow patterns (ci_test.cpp:692-768): e0, e5, uniform."""
    p = cases["h2o_cisd"]
    ref = O.Detset(p)
    g = gpu_detset(p)
    n = ref.n_dets
    for C in (np.eye(n)[:, [0]], np.eye(n)[:, [5]], np.full((n, 1), 1.0 / n)):
        S_slow = ref.sigma(C, slow=True)
        S = g.sigma(torch.from_numpy(C).cuda()).cpu().numpy()
        assert np.abs(S - S_slow).max() < 1e-13 * max(1.0, np.abs(S_slow).max())


def test_sigma_properties_medium():
    """Linearity and symmetry <X, HY> = <HX, Y> on FCI(12o, 6a6b) (853,776 dets)."""
    p = synthetic_fci(12, 6, 6, seed=21)
    g = gpu_detset(p)
    n = g.N_dets
    gen = torch.Generator(device="cuda").manual_seed(5)
    X = torch.randn(n, 2, device="cuda", dtype=torch.float64, generator=gen)
    Y = torch.randn(n, 2, device="cuda", dtype=torch.float64, generator=gen)
    HX, HY = g.sigma(X), g.sigma(Y)
    H_lin = g.sigma(0.3 * X - 1.7 * Y)
    assert (H_lin - (0.3 * HX - 1.7 * HY)).abs().max().item() <= 1e-12 * HX.abs().max().item()
    a = (X * HY).sum(0)
    b = (HX * Y).sum(0)
    assert ((a - b).abs() / a.abs().clamp_min(1.0)).max().item() < 1e-12
    # row-sampled exact check against the oracle
    ref = O.Detset(p, check_addressing=False)
    rows = np.random.default_rng(3).choice(n, size=2000, replace=False)
    Xh = X.cpu().numpy()
    S_rows = ref.sigma_rows(Xh, rows)
    assert np.abs(HX.cpu().numpy()[rows] - S_rows).max() <= SIGMA_RTOL_FP64 * np.abs(S_rows).max()


def test_sigma_fp32_full_ci_medium():
    """FP32 sigma of a full-CI space (transposed same-spin passes + alpha-beta scatter) against FP64."""
    from polyquant_gb300._lib import PQ_FP32

    p = synthetic_fci(12, 6, 6, seed=22)
    g = gpu_detset(p)
    gen = torch.Generator(device="cuda").manual_seed(6)
    for k in (1, 2, 4):
        X = torch.randn(g.N_dets, k, device="cuda", dtype=torch.float64, generator=gen)
        S64 = g.sigma(X)
        S32 = g.sigma(X, precision=PQ_FP32)
        assert (S32 - S64).abs().max().item() <= SIGMA_RTOL_FP32 * S64.abs().max().item()


@pytest.mark.parametrize("shape", [(10, 5, 4), (13, 6, 6), (7, 3, 3), (9, 1, 4)])
def test_sigma_fp32_tensor_core_alpha_beta_matches_scatter_path(monkeypatch, shape):
    """The FP32 full-CI sigma with its alpha-beta doubles on the tensor cores (FP16 hi/lo split, FP32
    accumulation) against the same sigma with the FP32 vector-atomic scatter (PQ_SIGMA32_NO_TC, read when a
    handle is created) and against FP64, for beta rows that fill 1 to 14 column tiles (the last one partial),
    fewer alpha singles than the GEMM's K = 64, and widths 1, 2, 4."""
    from polyquant_gb300._lib import PQ_FP32

    n, a, b = shape
    p = synthetic_fci(n, a, b, seed=30 + n)
    g_tc = gpu_detset(p)
    monkeypatch.setenv("PQ_SIGMA32_NO_TC", "1")
    g_sc = gpu_detset(p)
    monkeypatch.delenv("PQ_SIGMA32_NO_TC")
    gen = torch.Generator(device="cuda").manual_seed(n)
    for k in (1, 2, 4, 3):
        X = torch.randn(g_tc.N_dets, k, device="cuda", dtype=torch.float64, generator=gen)
        S64 = g_tc.sigma(X)
        S_tc = g_tc.sigma(X, precision=PQ_FP32)
        S_sc = g_sc.sigma(X, precision=PQ_FP32)
        scale = S64.abs().max().item()
        assert (S_tc - S64).abs().max().item() <= SIGMA_RTOL_FP32 * scale
        assert (S_sc - S64).abs().max().item() <= SIGMA_RTOL_FP32 * scale
        # the scaled split keeps 22 bits: no worse than FP32 arithmetic by more than a small factor
        assert (S_tc - S64).abs().max().item() <= 10 * max((S_sc - S64).abs().max().item(), 1e-7 * scale)
    # tiny and large magnitudes: the power-of-two scaling keeps the relative accuracy
    for f in (1e-30, 1e20):
        X = f * torch.randn(g_tc.N_dets, 2, device="cuda", dtype=torch.float64, generator=gen)
        S64 = g_tc.sigma(X)
        S_tc = g_tc.sigma(X, precision=PQ_FP32)
        assert (S_tc - S64).abs().max().item() <= SIGMA_RTOL_FP32 * S64.abs().max().item()
    g_tc.close()
    g_sc.close()


@pytest.mark.parametrize("shape", [(12, 6, 6, True), (13, 6, 5, True), (12, 6, 6, False)])
def test_sigma_fp32_same_spin_gemm_matches_gather_path(monkeypatch, shape):
    """The FP32 full-CI sigma with both same-spin double blocks as dense tensor-core GEMMs (FP16 hi/lo split,
    FP32 accumulation; 3 and 4 vectors use the 4-wide block) against the same sigma with the row-side gathers
    (PQ_SIGMA32_NO_SS, read when a handle is created) and against FP64: equal spin lists (the beta GEMM reuses
    the alpha matrix), unequal lists, and unrestricted integrals (two matrices); partial tiles in M, N and K."""
    from polyquant_gb300._lib import PQ_FP32

    n, a, b, restricted = shape
    p = synthetic_fci(n, a, b, seed=40 + n) if restricted else synthetic_unrestricted(n, a, b, seed=41)
    g_ss = gpu_detset(p)
    monkeypatch.setenv("PQ_SIGMA32_NO_SS", "1")
    g_ga = gpu_detset(p)
    monkeypatch.delenv("PQ_SIGMA32_NO_SS")
    gen = torch.Generator(device="cuda").manual_seed(n + a)
    for k in (4, 3):
        X = torch.randn(g_ss.N_dets, k, device="cuda", dtype=torch.float64, generator=gen)
        S64 = g_ss.sigma(X)
        S_ss = g_ss.sigma(X, precision=PQ_FP32)
        S_ga = g_ga.sigma(X, precision=PQ_FP32)
        scale = S64.abs().max().item()
        assert (S_ss - S64).abs().max().item() <= SIGMA_RTOL_FP32 * scale
        assert (S_ga - S64).abs().max().item() <= SIGMA_RTOL_FP32 * scale
        assert (S_ss - S64).abs().max().item() <= 10 * max((S_ga - S64).abs().max().item(), 1e-7 * scale)
    for f in (1e-30, 1e20):
        X = f * torch.randn(g_ss.N_dets, 4, device="cuda", dtype=torch.float64, generator=gen)
        S64 = g_ss.sigma(X)
        S_ss = g_ss.sigma(X, precision=PQ_FP32)
        assert (S_ss - S64).abs().max().item() <= SIGMA_RTOL_FP32 * S64.abs().max().item()
    g_ss.close()
    g_ga.close()


def test_davidson_h2o_energies(cases, h2o):
    """H2O/STO-3G CISD energies (calculation_test.cpp:253-260) and FCI vs the oracle's dense H."""
    r = h2o("library")
    p = cases["h2o_cisd"]
    g = gpu_detset(p)
    e, info = g.davidson(num_states=2, num_subspace_vec=20, convergence_E=1e-9, energy_shift=r["e_nuc"])
    assert info["converged"]
    assert abs(e[0] - (-75.01170307729812)) < 1e-6
    assert abs(e[1] - (-74.59209776692875)) < 1e-6
    w = np.linalg.eigvalsh(O.Detset(p).dense_ham()) + r["e_nuc"]
    assert np.abs(e - w[:2]).max() < ENERGY_TOL
    pf = cases["h2o_fci"]
    gf = gpu_detset(pf)
    ef, info = gf.davidson(num_states=1, num_subspace_vec=4, convergence_E=1e-9, energy_shift=r["e_nuc"])
    wf = np.linalg.eigvalsh(O.Detset(pf).dense_ham()) + r["e_nuc"]
    assert info["converged"] and abs(ef[0] - wf[0]) < ENERGY_TOL


def test_davidson_mixed_precision_reaches_fp64():
    from polyquant_gb300._lib import PQ_FP32

    p = synthetic_fci(8, 4, 4, seed=31)
    g = gpu_detset(p)
    e64, i64 = g.davidson(num_states=3, num_subspace_vec=6, convergence_E=1e-8)
    e32, i32 = g.davidson(num_states=3, num_subspace_vec=6, convergence_E=1e-8, precision=PQ_FP32)
    assert i64["converged"] and i32["converged"]
    assert np.abs(e32 - e64).max() < 1e-6
    assert i32["sigma_calls_fp32"] > 0
    ref = O.Detset(p)
    w = np.linalg.eigvalsh(ref.dense_ham())
    assert np.abs(e64 - w[:3]).max() < ENERGY_TOL


def test_invalid_problem_is_an_error():
    from polyquant_gb300._lib import PQError

    p = synthetic_fci(5, 3, 3, seed=0, ex=[3, 3, 6])
    with pytest.raises(PQError):
        gpu_detset(p)


def test_davidson_iteration_cap_reports_not_converged():
    """An iteration cap that is too small ends the solve with PQ_NOT_CONVERGED (the reference aborts,
    epci.cpp:620) and still returns the current Ritz values and residual."""
    from polyquant_gb300._lib import PQ_FP32, PQ_FP64

    p = synthetic_fci(8, 4, 4, seed=1)
    ds = gpu_detset(p)
    w = np.linalg.eigvalsh(O.Detset(p).dense_ham())
    for prec in (PQ_FP64, PQ_FP32):
        e, info = ds.davidson(num_states=2, num_subspace_vec=4, convergence_E=1e-10, iteration_max=3, precision=prec)
        assert not info["converged"]
        assert info["iterations"] == 3 and info["max_residual"] > 1e-10
        assert np.all(e >= w[:2] - 1e-9)  # Ritz values bound the eigenvalues from above
    ds.close()
