"""Parsing of the reference's JSON ci_keywords (calculation.cpp:274-389) on CPU."""
import json

import pytest

from polyquant_gb300 import ci_input

SAMPLE = {
    "molecule": {"symbols": ["H", "H", "O"], "molecular_charge": 0, "molecular_multiplicity": 1},
    "model": {"method": "CI"},
    "keywords": {
        "restricted": True,
        "ci_keywords": {
            "convergence_E": 1e-8, "num_states": 2, "num_subspace_vec": 20, "slow_diag": False,
            "excitation_level": [[2, 2, 4]], "frozen_core": [0], "deleted_virtual": [0],
            "build_matrix": False, "calc_s2": True, "fcidump_filename": "INTEGRALS",
            "spin_penalty_type": "first_order", "NO_states": [0, 1], "precision": "mixed",
        },
    },
}


def test_parse_values_and_unsupported(tmp_path):
    f = tmp_path / "in.json"
    f.write_text(json.dumps(SAMPLE))
    for src in (SAMPLE, str(f), json.dumps(SAMPLE)):
        kw = ci_input.parse(src)
        assert kw.convergence_E == 1e-8 and kw.num_states == 2 and kw.num_subspace_vec == 20
        assert kw.excitation_levels(1) == [[2, 2, 4]]
        assert kw.frozen_core == [0] and kw.deleted_virtual == [0]
        assert not kw.build_matrix and kw.calc_s2 and kw.precision == "mixed"
        assert kw.fcidump_filename == "INTEGRALS"
        assert kw.NO_states == [0, 1]
        assert kw.unsupported == ["spin_penalty_type"]


def test_defaults_match_the_reference():
    kw = ci_input.parse({"keywords": {"ci_keywords": {}}})
    # epci.hpp:113-122, determinant_set.hpp:195-196
    assert (kw.convergence_E, kw.num_states, kw.num_subspace_vec, kw.iteration_max) == (1e-6, 1, 5, 500)
    assert kw.build_matrix and not kw.exact_diag and not kw.slow_diag
    assert kw.NO_states == [0]  # calculation.cpp:335-345
    assert kw.excitation_levels(2) is None and kw.precision == "fp64"


def test_scalar_excitation_level_and_errors():
    kw = ci_input.parse({"keywords": {"ci_keywords": {"excitation_level": 2}}})
    assert kw.excitation_levels(2) == [[2, 2, 2], [2, 2, 2]]
    with pytest.raises(ValueError):
        ci_input.parse({"keywords": {"ci_keywords": {"frozen_core": True}}})
    with pytest.raises(ValueError):
        ci_input.parse({"keywords": {"ci_keywords": {"precision": "fp16"}}})
    kw = ci_input.parse({"keywords": {"ci_keywords": {"excitation_level": [[1, 1, 2]]}}})
    with pytest.raises(ValueError):
        kw.excitation_levels(2)
