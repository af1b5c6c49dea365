"""The reference's JSON ``ci_keywords`` on top of the GB300 path.

``parse`` reads ``keywords.ci_keywords`` of a polyquant input (dict or file),
with the keys, value forms and defaults of the reference
(src/calculation/calculation.cpp:274-389; defaults src/ci/epci.hpp:113-122,
src/ci/determinant_set.hpp:195-196), plus three keys of this implementation:
``precision`` ("fp64" or "mixed"), ``batch`` and ``autotune``.  Keys the
GB300 path does not implement (spin penalties, symmetrised natural orbitals,
printing thresholds) are collected in ``CIKeywords.unsupported`` instead of being
silently dropped.

``run`` solves one CI problem as ``POLYQUANT_EPCI::run`` would
(src/ci/epci.cpp:575-686): the explicit sparse Hamiltonian when
``build_matrix`` is set (the reference default), dense diagonalisation of it
for ``exact_diag`` (ignored without ``build_matrix``, as in the reference),
block Davidson otherwise, <S^2> per state and species for
``calc_s2``, and the natural spin orbitals of the ``NO_states`` (default
[0]; calculate_NOs, epci.cpp:200-318) in the basis of the caller's SCF
orbitals, or in the MO basis when none are given.
The integrals come from the caller or from the FCIDUMP file named by
``fcidump_filename``.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from typing import List, Optional, Union

import numpy as np

from .detset import INT_MAX

SUPPORTED = {"convergence_E", "num_states", "num_subspace_vec", "iteration_max", "build_matrix", "exact_diag",
             "slow_diag", "excitation_level", "max_collective_excitation_level", "screening_threshold",
             "frozen_core", "deleted_virtual", "calc_s2", "NO_states", "fcidump_filename", "precision", "batch",
             "autotune"}


@dataclass
class CIKeywords:
    convergence_E: float = 1e-6
    num_states: int = 1
    num_subspace_vec: int = 5
    iteration_max: int = 500
    build_matrix: bool = True
    exact_diag: bool = False
    slow_diag: bool = False
    excitation_level: Optional[Union[int, List[List[int]]]] = None
    max_collective_excitation_level: int = INT_MAX
    screening_threshold: float = 0.0
    frozen_core: List[int] = field(default_factory=list)
    deleted_virtual: List[int] = field(default_factory=list)
    calc_s2: bool = False
    NO_states: List[int] = field(default_factory=lambda: [0])
    fcidump_filename: Optional[str] = None
    precision: str = "fp64"
    batch: bool = False
    autotune: bool = True
    unsupported: List[str] = field(default_factory=list)

    def excitation_levels(self, n_species: int) -> Optional[List[List[int]]]:
        """[[alpha_max, beta_max, total_max] per species]; a scalar applies to every entry of every species
        (calculation.cpp:346-362)."""
        e = self.excitation_level
        if e is None:
            return None
        if isinstance(e, (int, np.integer)):
            return [[int(e)] * 3 for _ in range(n_species)]
        if len(e) < n_species:
            raise ValueError(f"excitation_level lists {len(e)} species, the problem has {n_species}")
        return [[int(x) for x in e[s][:3]] for s in range(n_species)]


def parse(data: Union[dict, str]) -> CIKeywords:
    """``keywords.ci_keywords`` of a polyquant input (a dict, a JSON string or a file name)."""
    if isinstance(data, str):
        if data.lstrip().startswith("{"):
            data = json.loads(data)
        else:
            with open(data) as f:
                data = json.load(f)
    ck = data.get("keywords", {}).get("ci_keywords", {})
    kw = CIKeywords()
    for k, v in ck.items():
        if k not in SUPPORTED:
            kw.unsupported.append(k)
            continue
        if k == "NO_states":
            v = [int(x) for x in v] if isinstance(v, list) else [0]  # calculation.cpp:335-345
        elif k in ("frozen_core", "deleted_virtual"):
            if isinstance(v, bool):
                raise ValueError(f"ci_keywords.{k} must be a list of numbers")  # as calculation.cpp:374-389
            v = [int(x) for x in v]
        elif k == "precision":
            if v not in ("fp64", "mixed"):
                raise ValueError("ci_keywords.precision must be 'fp64' or 'mixed'")
        elif k in ("convergence_E", "screening_threshold"):
            v = float(v)
        elif k in ("num_states", "num_subspace_vec", "iteration_max", "max_collective_excitation_level"):
            v = int(v)
        elif k in ("build_matrix", "exact_diag", "slow_diag", "calc_s2", "batch", "autotune"):
            v = bool(v)
        setattr(kw, k, v)
    return kw


def run(kw: CIKeywords, problem: Optional[dict] = None, e_const: float = 0.0, mo_coeff=None) -> dict:
    """Solve one CI problem.  ``problem``: POLYQUANT_DETSET keyword arguments (integrals in the reference layout);
    when None, the integrals come from ``kw.fcidump_filename``.  ``mo_coeff``: optional [species][spin] SCF
    orbitals (n_ao x n_mo, frozen-core orbitals first as ``kw.frozen_core`` says) for the natural orbitals.
    Returns energies (+ e_const), <S^2> when requested, natural orbitals and the solver report."""
    import torch

    from . import fcidump
    from ._lib import PQ_FP32, PQ_FP64
    from .detset import POLYQUANT_DETSET

    if problem is None:
        if not kw.fcidump_filename:
            raise ValueError("no integrals: pass a problem or set ci_keywords.fcidump_filename")
        problem, e_const = fcidump.problem_from_fcidump(kw.fcidump_filename)
    problem = dict(problem)
    lv = kw.excitation_levels(len(problem["n_orb"]))
    if lv is not None:
        problem["excitation_level"] = lv
    if kw.max_collective_excitation_level != INT_MAX:
        problem["max_collective_excitation_level"] = kw.max_collective_excitation_level
    ds = POLYQUANT_DETSET(**problem)
    k = min(kw.num_states, ds.N_dets)
    out = {"n_dets": ds.N_dets, "method": None}
    try:
        if kw.build_matrix:
            out["nnz"] = ds.create_ham(screening_threshold=kw.screening_threshold, use_for_sigma=True)
        if kw.exact_diag and kw.build_matrix:  # exact_diag acts only on the explicit matrix (epci.cpp:605-633)
            rp, col, val = ds.ham_csr(upper=False)
            H = np.zeros((ds.N_dets, ds.N_dets))
            for i in range(ds.N_dets):
                H[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
            w, V = np.linalg.eigh(H)
            e, vecs = w[:k], torch.from_numpy(np.ascontiguousarray(V[:, :k])).cuda()
            out["method"] = "exact_diag"
        else:
            prec = PQ_FP32 if kw.precision == "mixed" else PQ_FP64
            e, vecs, info = ds.davidson(num_states=k, num_subspace_vec=max(kw.num_subspace_vec, k),
                                        iteration_max=kw.iteration_max, convergence_E=kw.convergence_E,
                                        precision=prec, return_vectors=True)
            out["method"] = "davidson"
            out["report"] = info
        out["energies"] = (np.asarray(e) + e_const).tolist()
        if kw.calc_s2:
            out["s2"] = ds.s2(vecs).tolist()
        states = [st for st in kw.NO_states if 0 <= st < k]
        if states:
            from .natural_orbitals import calculate_NOs

            if mo_coeff is None:
                C_combined, fc = [[np.eye(n)] for n in ds.n_orb], None
            else:
                C_combined = mo_coeff
                fc = list(kw.frozen_core) + [0] * (ds.n_species - len(kw.frozen_core))
            out["natural_orbitals"] = calculate_NOs(ds, vecs, C_combined, NO_states=states, frozen_core=fc)
    finally:
        ds.close()
    return out
