"""pq_ci_sigma_host (operator* with host buffers) against the device entry point and the oracle: page-locked
buffers read and written in place by the layout-conversion kernels, the same buffers through the staged copies
(PQ_SIGMA_HOST_STAGED), and pageable buffers; padded leading dimensions, 5 vectors (two interleaved blocks),
FP64 and FP32, one species and an electron + positron space.  The three host routes run the same kernels on
the same values as the device entry point, so their results are bit-identical to it."""
import ctypes

import numpy as np
import pytest

import oracle as O
from cases import batch_dict, h2o_problem, synthetic_ep

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = {
    "h2o_cisd": lambda h2o: h2o_problem(h2o("library"), [2, 2, 2]),
    "ep_coll3_2pos": lambda h2o: synthetic_ep(5, 2, 2, 4, 1, 1, seed=4, max_coll=3),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request, h2o):
    from polyquant_gb300.detset import POLYQUANT_DETSET

    p = CASES[request.param](h2o)
    g = POLYQUANT_DETSET(**batch_dict(p))
    yield request.param, p, g
    g.close()


def _host_sigma(g, C, S, ld, nvec, prec):
    from polyquant_gb300 import _lib

    ptr = (lambda a: ctypes.c_void_p(a.data_ptr())) if isinstance(C, torch.Tensor) else (lambda a: a.ctypes.data)
    _lib.check(_lib.load().pq_ci_sigma_host(g._h, ptr(C), ld, nvec, ptr(S), ld, prec), "pq_ci_sigma_host")


@pytest.mark.parametrize("prec_name", ["fp64", "fp32"])
def test_host_routes_match_device_and_oracle(case, prec_name, monkeypatch):
    from polyquant_gb300 import _lib

    name, p, g = case
    prec = _lib.PQ_FP64 if prec_name == "fp64" else _lib.PQ_FP32
    n, nvec = g.N_dets, 5
    ld = n + 7  # padded leading dimension
    rng = np.random.default_rng(2)
    Cn = np.zeros((nvec, ld))
    Cn[:, :n] = rng.standard_normal((nvec, n))
    # device entry point on the same column-major block
    Cd = torch.from_numpy(Cn).cuda()
    Sd = torch.zeros_like(Cd)
    _lib.check(_lib.load().pq_ci_sigma(g._h, ctypes.c_void_p(Cd.data_ptr()), ld, nvec, ctypes.c_void_p(Sd.data_ptr()),
                                       ld, prec), "pq_ci_sigma")
    S_dev = Sd.cpu().numpy()[:, :n]
    # page-locked, in place
    Cp = torch.from_numpy(Cn).pin_memory()
    Sp = torch.zeros((nvec, ld), dtype=torch.float64).pin_memory()
    assert Cp.is_pinned() and Sp.is_pinned()
    _host_sigma(g, Cp, Sp, ld, nvec, prec)
    assert np.array_equal(Sp.numpy()[:, :n], S_dev), name
    assert np.all(Sp.numpy()[:, n:] == 0.0)  # the padding rows are not written
    # page-locked, staged copies
    Sp.zero_()
    monkeypatch.setenv("PQ_SIGMA_HOST_STAGED", "1")
    _host_sigma(g, Cp, Sp, ld, nvec, prec)
    monkeypatch.delenv("PQ_SIGMA_HOST_STAGED")
    assert np.array_equal(Sp.numpy()[:, :n], S_dev), name
    # pageable
    Sn = np.zeros((nvec, ld))
    _host_sigma(g, Cn, Sn, ld, nvec, prec)
    assert np.array_equal(Sn[:, :n], S_dev), name
    # and the oracle
    S_ref = O.Detset(p).sigma(Cn[:, :n].T.copy()).T
    tol = 1e-10 if prec == _lib.PQ_FP64 else 2e-5
    assert np.abs(S_dev - S_ref).max() <= tol * np.abs(S_ref).max(), name
