"""Parity at the exact sizes the benchmark times, against the oracle (the reference's fast-vs-slow sigma
self-test, ci_test.cpp:692-852, is the template: one sigma implementation checked against another on the same
vectors).

* FCI(16 orbitals, 8a+8b): 165,636,900 determinants, 4 roots, synthetic integrals of seed 0 -- the FP64 and
  FP32 sigma on 4,096 random rows plus the first and last rows of the space, and the diagonal on those rows,
  against the oracle's gather sigma (the reference's element formulas, direct_singleparticle.cpp:238-372).
* AO->MO at N_AO = N_MO = 256 with L = 1024 factors: 256 sampled rows (ij|*) of every mode against the
  factorized numpy restatement of transform_mo_2_body_integrals (integral.cpp:207-477).
* The electron-positron product space of 1a1b electrons in 60 orbitals x 1 positron in 40 orbitals
  (144,000 determinants, 3 roots): the FP64 and FP32 sigma on every row against the oracle's restatement of
  sigma_two_species_class_singleshot (direct_mixedparticle.cpp:269-611).

Tolerances are those of the smaller parity tests: FP64 sigma 1e-10, FP32 sigma 2e-5 relative to max |sigma|;
AO->MO FP64 1e-11, BF16x3 2e-4, TF32x3 2e-5 relative to max |(ij|kl)|.
"""
import numpy as np
import pytest

import oracle as O
from polyquant_gb300 import synthetic

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SIGMA_RTOL_FP64 = 1e-10
SIGMA_RTOL_FP32 = 2e-5
AO2MO_TOL = {"fp64": 1e-11, "bf16x3": 2e-4, "tf32x3": 2e-5}


def test_fci16_sigma_rows_and_diagonal_vs_oracle():
    from polyquant_gb300._lib import PQ_FP32
    from polyquant_gb300.detset import POLYQUANT_DETSET

    n_orb, ne, roots = 16, 8, 4
    h, eri = synthetic.fci_integrals(n_orb, seed=0)
    ex = [ne, ne, 2 * ne]
    g = POLYQUANT_DETSET([n_orb], [ne], [ne], [[h, h]], {(0, 0, 0, 0): eri}, [ex])
    n = g.N_dets
    assert n == 165_636_900
    # (roots x n) row-major == the column-major (n x roots) block the reference passes
    Ct = np.random.default_rng(7).standard_normal((roots, n))
    X = torch.from_numpy(Ct).cuda().t()
    rows = np.concatenate([[0, 1, 12_869, n // 2, n - 1],
                           np.random.default_rng(8).choice(n, size=4096, replace=False)])
    rows_t = torch.from_numpy(rows).cuda()
    S64 = g.sigma(X)[rows_t].cpu().numpy()
    S32 = g.sigma(X, precision=PQ_FP32)[rows_t].cpu().numpy()
    D = g.diagonal()[rows_t].cpu().numpy()
    del X
    g.close()
    torch.cuda.empty_cache()

    ref = O.Detset(O.CIProblem([n_orb], [ne], [ne], [[h, h]], {(0, 0, 0, 0): eri}, [ex]), check_addressing=False)
    S_ref = ref.sigma_rows(Ct.T, rows)  # (n x roots) Fortran-ordered view of the same values
    D_ref = ref.diagonal()[rows]
    scale = np.abs(S_ref).max()
    assert np.abs(S64 - S_ref).max() <= SIGMA_RTOL_FP64 * scale
    assert np.abs(S32 - S_ref).max() <= SIGMA_RTOL_FP32 * scale
    assert np.abs(D - D_ref).max() <= 1e-12 * np.abs(D_ref).max()


@pytest.fixture(scope="module")
def ao2mo_n256():
    n, L = 256, 1024
    Bp = synthetic.ao_eri_pairs(n, seed=0, L=L)
    C = synthetic.mo_coefficients(n, n, seed=1)
    rows = np.random.default_rng(3).choice(n * (n + 1) // 2, size=256, replace=False)
    ref = O.ao2mo_rows_factorized(Bp, C, rows)
    return Bp, C, rows, ref


@pytest.mark.parametrize("mode", ["fp64", "bf16x3", "tf32x3"])
def test_ao2mo_n256_rows_vs_oracle(ao2mo_n256, mode):
    from polyquant_gb300._lib import PQ_XFORM_BF16X3, PQ_XFORM_FP64, PQ_XFORM_TF32X3
    from polyquant_gb300.integral import ao2mo

    Bp, C, rows, ref = ao2mo_n256
    Bd = torch.from_numpy(Bp).cuda()
    M = Bd.t() @ Bd  # the pair matrix of the AO integrals, as the benchmark forms it
    del Bd
    mask = torch.ones(M.shape[0], M.shape[0], dtype=torch.bool, device="cuda").tril_()
    packed = torch.masked_select(M, mask)
    del M, mask
    mode_id = {"fp64": PQ_XFORM_FP64, "bf16x3": PQ_XFORM_BF16X3, "tf32x3": PQ_XFORM_TF32X3}[mode]
    out = ao2mo(packed, torch.from_numpy(C).cuda(), mode=mode_id)
    got = out[torch.from_numpy(rows).cuda()].cpu().numpy()
    del out, packed
    from polyquant_gb300 import _lib

    _lib.load().pq_ao2mo_release_workspace()
    torch.cuda.empty_cache()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < AO2MO_TOL[mode], err


def test_psh_like_product_space_sigma_vs_oracle():
    from polyquant_gb300._lib import PQ_FP32
    from polyquant_gb300.detset import POLYQUANT_DETSET

    n_e, n_p = 60, 40
    h_e, h_p, ee, pp, ep = synthetic.ep_integrals(n_e, n_p, seed=0)
    args = ([n_e, n_p], [1, 1], [1, 0], [[h_e, h_e], [h_p, h_p]], {(0, 0, 0, 0): ee, (1, 0, 1, 0): pp, (0, 0, 1, 0): ep},
            [[1, 1, 2], [1, 0, 1]])
    g = POLYQUANT_DETSET(*args, restricted=[1, 1], charge=[-1.0, 1.0])
    assert g.N_dets == 144_000
    C = np.random.default_rng(4).standard_normal((g.N_dets, 3))
    Xd = torch.from_numpy(C).cuda()
    S64 = g.sigma(Xd).cpu().numpy()
    S32 = g.sigma(Xd, precision=PQ_FP32).cpu().numpy()
    g.close()
    ref = O.Detset(O.CIProblem(*args, restricted=[1, 1], charge=[-1.0, 1.0]))
    S_ref = ref.sigma(C)
    scale = np.abs(S_ref).max()
    assert np.abs(S64 - S_ref).max() <= SIGMA_RTOL_FP64 * scale
    assert np.abs(S32 - S_ref).max() <= SIGMA_RTOL_FP32 * scale
