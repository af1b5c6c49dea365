"""JSON ci_keywords + FCIDUMP -> GPU CI, against the reference's H2O/STO-3G CISD energies
(tests/integration_tests/calculation/calculation_test.cpp:259-260, tolerance 1e-6)."""
import numpy as np
import pytest

from cases import batch_dict, h2o_problem
from polyquant_gb300 import ci_input, fcidump

pytestmark = pytest.mark.gpu
E_CISD = [-75.01170307729812, -74.59209776692875]


@pytest.fixture(scope="module")
def integrals(h2o, tmp_path_factory):
    r = h2o("library")
    p = h2o_problem(r, [2, 2, 2])
    d = batch_dict(p)
    base = str(tmp_path_factory.mktemp("fcidump") / "INTEGRALS")
    names = fcidump.dump_problem(base, ["e"], h1=d["h1"], eri=d["eri"], n_part=[10], ms2=[0], restricted=[1],
                                 e_const=r["e_nuc"])
    return names[0]


@pytest.mark.parametrize("extra", [{"build_matrix": True}, {"build_matrix": False},
                                   {"build_matrix": True, "exact_diag": True}, {"build_matrix": False,
                                                                               "precision": "mixed"}])
def test_cisd_from_json_and_fcidump(integrals, extra):
    ck = {"convergence_E": 1e-8, "num_states": 2, "num_subspace_vec": 6, "excitation_level": [[2, 2, 2]],
          "calc_s2": True, "fcidump_filename": integrals}
    ck.update(extra)
    kw = ci_input.parse({"keywords": {"ci_keywords": ck}})
    out = ci_input.run(kw)
    assert out["n_dets"] == 141
    assert np.abs(np.array(out["energies"]) - E_CISD).max() < 1e-6
    assert abs(out["s2"][0]) < 1e-6  # closed-shell ground state: a singlet
    occ = out["natural_orbitals"]["occ_nso"][0][0][0]  # state 0, electrons, alpha (MO basis)
    assert abs(occ.sum() - 5) < 1e-8 and np.all(np.diff(occ) <= 0)


@pytest.mark.parametrize("extra", [{"build_matrix": True}, {"build_matrix": True, "exact_diag": True},
                                   {"build_matrix": False}])
def test_electron_positron_from_json(extra):
    import oracle as O
    from cases import synthetic_ep

    p = synthetic_ep(5, 2, 2, 4, 1, 0, seed=7)
    w = np.linalg.eigvalsh(O.Detset(p).dense_ham())
    ck = {"convergence_E": 1e-9, "num_states": 2, "num_subspace_vec": 6, "calc_s2": True}
    ck.update(extra)
    out = ci_input.run(ci_input.parse({"keywords": {"ci_keywords": ck}}), problem=batch_dict(p), e_const=0.5)
    assert ("nnz" in out) == extra["build_matrix"]
    assert np.abs(np.array(out["energies"]) - 0.5 - w[:2]).max() < 1e-8
    assert np.array(out["s2"]).shape == (2, 2)
