"""Host-side mirror of polyquant's determinant-set operator on the GB300 library.

``POLYQUANT_DETSET`` keeps the reference's operator interface
(src/ci/determinant_set.hpp:120-170): ``rows()``, ``cols()``, ``op(i, j)`` /
``Slater_Condon(i, j)`` (any element, slater_condon.cpp:4-100), ``op * X`` / ``op @ X`` (sigma,
direct.cpp:5-18) and ``create_sigma(sigma, C)`` (direct.cpp:21-33).  Every
operation calls the C ABI of libpq_gb300.so; there is no CPU path.

Inputs follow the reference conventions: MO one-body integrals per species and
spin, MO ERI blocks (npair_a x npair_b, [idx2(i,j), idx2(k,l)]), excitation
levels {alpha, beta, total} per species and the collective limit.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Sequence

import numpy as np

from . import _lib
from ._lib import PQ_FP32, PQ_FP64, check  # noqa: F401  (PQ_FP32 re-exported for callers)

INT_MAX = 2 ** 31 - 1


def _torch():
    import torch

    return torch


def make_desc(n_orb: Sequence[int], n_alpha: Sequence[int], n_beta: Sequence[int], h1, eri: Dict,
              excitation_level: Sequence[Sequence[int]], restricted: Sequence[int] = None,
              charge: Sequence[float] = None, max_collective_excitation_level: int = INT_MAX):
    """pq_ci_desc for one problem plus the Fortran-ordered integral arrays it points to (keep them alive
    until the create call returns)."""
    ns = len(n_orb)
    restricted = list(restricted) if restricted is not None else [1] * ns
    charge = list(charge) if charge is not None else [-1.0] * ns
    d = _lib.PQDesc()
    d.n_species = ns
    keep = []
    for s in range(ns):
        d.n_orb[s] = int(n_orb[s])
        d.n_alpha[s] = int(n_alpha[s])
        d.n_beta[s] = int(n_beta[s])
        d.restricted[s] = int(restricted[s])
        d.charge[s] = float(charge[s])
        for t in range(3):
            d.ex_level[s][t] = int(excitation_level[s][t])
        nb = 1 if restricted[s] else 2
        for sp in range(2):
            m = np.asfortranarray(np.asarray(h1[s][sp % nb] if len(h1[s]) > sp % nb else h1[s][0],
                                             dtype=np.float64))
            keep.append(m)
            d.h1[s][sp] = m.ctypes.data
    d.max_collective = int(max_collective_excitation_level)
    for a in range(ns):
        for sa in range(2):
            for b in range(a, ns):
                for sb in range(2):
                    key = (a, sa % (1 if restricted[a] else 2), b, sb % (1 if restricted[b] else 2))
                    m = eri.get(key)
                    if m is None and a == b and (a, key[3], a, key[1]) in eri:
                        m = np.asarray(eri[(a, key[3], a, key[1])]).T
                    if m is None:
                        continue
                    m = np.asfortranarray(np.asarray(m, dtype=np.float64))
                    keep.append(m)
                    d.eri[a][sa][b][sb] = m.ctypes.data
    return d, keep


class POLYQUANT_DETSET:
    """Determinant space + Hamiltonian operator built on the GPU.

    Parameters mirror ``pq_ci_desc``: ``h1[s][spin]`` (n x n) and
    ``eri[(a, sa, b, sb)]`` (npair_a x npair_b) as numpy arrays; restricted
    species need only spin index 0.
    """

    Scalar = float

    def __init__(self, n_orb: Sequence[int], n_alpha: Sequence[int], n_beta: Sequence[int], h1, eri: Dict,
                 excitation_level: Sequence[Sequence[int]] = None, restricted: Sequence[int] = None,
                 charge: Sequence[float] = None, max_collective_excitation_level: int = INT_MAX, stream=None,
                 selected_strings: Sequence[Sequence] = None):
        """``selected_strings[s][spin]`` (optional): occupation masks (bit o = orbital o) of a selected-string
        space (``pq_ci_create_selected``, an extension: the determinants are the full product of these lists
        and ``excitation_level`` is ignored)."""
        L = _lib.load()
        ns = len(n_orb)
        if excitation_level is None:
            if selected_strings is None:
                raise ValueError("excitation_level is required unless selected_strings is given")
            excitation_level = [[0, 0, 0]] * ns
        d, self._keep = make_desc(n_orb, n_alpha, n_beta, h1, eri, excitation_level, restricted, charge,
                                  max_collective_excitation_level)
        self._desc = d
        self._stream = stream
        h = ctypes.c_void_p()
        if selected_strings is None:
            check(L.pq_ci_create(ctypes.byref(d), ctypes.c_void_p(stream or 0), ctypes.byref(h)), "pq_ci_create")
        else:
            lists = [np.ascontiguousarray(np.asarray(selected_strings[s][sp], dtype=np.uint64))
                     for s in range(ns) for sp in range(2)]
            ptrs = (ctypes.c_void_p * len(lists))(*[a.ctypes.data for a in lists])
            counts = (ctypes.c_int64 * len(lists))(*[len(a) for a in lists])
            check(L.pq_ci_create_selected(ctypes.byref(d), ptrs, counts, ctypes.c_void_p(stream or 0),
                                          ctypes.byref(h)), "pq_ci_create_selected")
            del lists
        self._h = h
        self._keep = []  # integrals were copied to the device
        n = ctypes.c_int64()
        check(L.pq_ci_num_dets(self._h, ctypes.byref(n)))
        self.N_dets = n.value
        self.n_species = ns
        self.n_orb = [int(d.n_orb[s]) for s in range(ns)]
        self.n_alpha = [int(d.n_alpha[s]) for s in range(ns)]
        self.n_beta = [int(d.n_beta[s]) for s in range(ns)]
        self.restricted = [int(d.restricted[s]) for s in range(ns)]
        self.excitation_level = [[int(x) for x in d.ex_level[s]] for s in range(ns)]
        self._diag = None

    # ---- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            _lib.load().pq_ci_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- Spectra operator concept ------------------------------------------
    def rows(self) -> int:
        return self.N_dets

    def cols(self) -> int:
        return self.N_dets

    def diagonal(self):
        """Device tensor of H_II (torch.float64, cuda)."""
        torch = _torch()
        if self._diag is None:
            out = torch.empty(self.N_dets, dtype=torch.float64, device="cuda")
            check(_lib.load().pq_ci_diag(self._h, ctypes.c_void_p(out.data_ptr())), "pq_ci_diag")
            self._diag = out
        return self._diag

    def _check_index(self, what: str, k) -> int:
        if isinstance(k, (bool, np.bool_)) or not isinstance(k, (int, np.integer)):
            raise TypeError(f"{what}: determinant index must be an integer, got {type(k).__name__}")
        if not 0 <= int(k) < self.N_dets:
            raise IndexError(f"{what}: determinant index {int(k)} outside 0..{self.N_dets - 1}")
        return int(k)

    def __call__(self, i: int, j: int) -> float:
        """H_ij, as the reference's operator()(i, j) = Slater_Condon(i, j) (determinant_set.hpp:139,
        slater_condon.cpp:4-100): exact FP64 for any pair, from the connections of determinant i
        (pq_ci_element), whatever an explicit matrix built with a screening threshold has pruned."""
        i, j = self._check_index("operator()", i), self._check_index("operator()", j)
        v = ctypes.c_double()
        check(_lib.load().pq_ci_element(self._h, i, j, ctypes.byref(v)), "pq_ci_element")
        return v.value

    Slater_Condon = __call__

    def elements(self, I, J) -> np.ndarray:
        """H_IJ for arrays of index pairs (one library call)."""
        I = np.ascontiguousarray(np.asarray(I, dtype=np.int64).reshape(-1))
        J = np.ascontiguousarray(np.asarray(J, dtype=np.int64).reshape(-1))
        if I.shape != J.shape:
            raise ValueError("elements: I and J differ in length")
        bad = (I < 0) | (I >= self.N_dets) | (J < 0) | (J >= self.N_dets)
        if bad.any():
            k = int(np.argmax(bad))
            raise IndexError(f"elements: pair ({I[k]}, {J[k]}) outside 0..{self.N_dets - 1}")
        out = np.zeros(I.shape[0])
        check(_lib.load().pq_ci_elements(self._h, I.shape[0], I.ctypes.data, J.ctypes.data, out.ctypes.data),
              "pq_ci_elements")
        return out

    def sigma(self, C, precision: int = PQ_FP64):
        """sigma = H C.  C: torch CUDA tensor (n_dets,) or (n_dets, k) float64, or a numpy array."""
        if isinstance(C, np.ndarray):
            return self._sigma_host(C, precision)
        torch = _torch()
        squeeze = C.dim() == 1
        X = C.reshape(self.N_dets, -1)
        # column-major n x k == row-major k x n
        Xc = X.t().contiguous().to(torch.float64)
        S = torch.empty_like(Xc)
        k = Xc.shape[0]
        check(_lib.load().pq_ci_sigma(self._h, ctypes.c_void_p(Xc.data_ptr()), self.N_dets, k,
                                      ctypes.c_void_p(S.data_ptr()), self.N_dets, precision), "pq_ci_sigma")
        out = S.t()
        return out.reshape(-1) if squeeze else out

    def _sigma_host(self, C: np.ndarray, precision: int):
        squeeze = C.ndim == 1
        X = np.asfortranarray(np.asarray(C, dtype=np.float64).reshape(self.N_dets, -1))
        S = np.zeros_like(X, order="F")
        check(_lib.load().pq_ci_sigma_host(self._h, X.ctypes.data, self.N_dets, X.shape[1], S.ctypes.data,
                                           self.N_dets, precision), "pq_ci_sigma_host")
        return S.reshape(-1) if squeeze else S

    def __mul__(self, X):
        return self.sigma(X)

    __matmul__ = __mul__

    def create_sigma(self, sigma, C):
        """In-place form of the reference's create_sigma(sigma, C) (sigma is overwritten)."""
        sigma[...] = self.sigma(C)
        return sigma

    # ---- strings / determinants ----------------------------------------------
    def strings(self, species: int, spin: int) -> np.ndarray:
        L = _lib.load()
        n = ctypes.c_int64()
        nw = ctypes.c_int32()
        check(L.pq_ci_strings(self._h, species, spin, None, ctypes.byref(n), ctypes.byref(nw)))
        out = np.zeros((n.value, nw.value), dtype=np.uint64)
        check(L.pq_ci_strings(self._h, species, spin, out.ctypes.data, ctypes.byref(n), ctypes.byref(nw)))
        return out

    def det_unfold(self) -> np.ndarray:
        """(N_dets, 2 * n_species) string indices of every determinant, in determinant order."""
        out = np.zeros((self.N_dets, 2 * self.n_species), dtype=np.int32)
        check(_lib.load().pq_ci_det_unfold(self._h, out.ctypes.data))
        return out

    def det_idx_unfold(self, det_idx: int):
        """String indices of one determinant, as the reference's det_idx_unfold (determinant_creation.cpp:378-388),
        which raises for an index outside the list where the reference aborts."""
        if not 0 <= det_idx < self.N_dets:
            raise IndexError(f"det_idx_unfold: {det_idx} outside 0..{self.N_dets - 1}")
        if getattr(self, "_unfold", None) is None:
            self._unfold = self.det_unfold()
        return [int(x) for x in self._unfold[det_idx]]

    def get_det(self, idx_part: int, idx_spin: int, i: int) -> np.ndarray:
        """Words of string i of a species and spin in the reference layout (word 0 = highest orbitals),
        as get_det (determinant_creation.cpp:390)."""
        return self.strings(idx_part, idx_spin)[i]

    # ---- eigen-solver ----------------------------------------------------------
    # ---- explicit Hamiltonian (create_ham, explicit_ham.cpp:51-84) -----------
    def create_ham(self, screening_threshold: float = 0.0, use_for_sigma: bool = True) -> int:
        """Build the sparse H on the device; FP64 sigma then multiplies with it. Returns stored entries."""
        nnz = ctypes.c_int64()
        check(_lib.load().pq_ci_ham_build(self._h, screening_threshold, 1 if use_for_sigma else 0,
                                          ctypes.byref(nnz)), "pq_ci_ham_build")
        return nnz.value

    def ham_csr(self, upper: bool = True):
        """(row_ptr, col, val) numpy arrays; upper=True is the reference's upper-triangle storage."""
        L = _lib.load()
        nnz = ctypes.c_int64()
        check(L.pq_ci_ham_csr(self._h, 1 if upper else 0, ctypes.byref(nnz), None, None, None), "pq_ci_ham_csr")
        rp = np.zeros(self.N_dets + 1, dtype=np.int64)
        col = np.zeros(max(nnz.value, 1), dtype=np.int32)
        val = np.zeros(max(nnz.value, 1), dtype=np.float64)
        check(L.pq_ci_ham_csr(self._h, 1 if upper else 0, ctypes.byref(nnz), rp.ctypes.data, col.ctypes.data,
                              val.ctypes.data), "pq_ci_ham_csr")
        return rp, col[:nnz.value], val[:nnz.value]

    # ---- properties of CI vectors (s2.cpp, rdm1.cpp) -------------------------
    def s2(self, C) -> np.ndarray:
        """<S^2> of each column of C (torch CUDA tensor (n_dets, k) or (n_dets,)): shape (k,) for one species,
        (k, n_species) for two."""
        torch = _torch()
        X = C.reshape(self.N_dets, -1).t().contiguous().to(torch.float64)
        out = np.zeros((X.shape[0], self.n_species))
        check(_lib.load().pq_ci_s2(self._h, ctypes.c_void_p(X.data_ptr()), self.N_dets, X.shape[0], out.ctypes.data),
              "pq_ci_s2")
        return out[:, 0] if self.n_species == 1 else out

    def rdm1(self, c, spin: int = 0, species: int = 0) -> np.ndarray:
        """One-particle density matrix (n_orb x n_orb) of the state vector c for one species and spin."""
        torch = _torch()
        x = c.reshape(-1).contiguous().to(torch.float64)
        n = self._desc.n_orb[species]
        out = np.zeros((n, n), order="F")
        check(_lib.load().pq_ci_rdm1(self._h, ctypes.c_void_p(x.data_ptr()), species, spin, out.ctypes.data),
              "pq_ci_rdm1")
        return out

    # the reference's names and argument order for the same two properties
    def evaluate_s2(self, C) -> np.ndarray:
        """S_squared (n_states x n_species) as POLYQUANT_DETSET::evaluate_s2 fills it (s2.cpp:4-123)."""
        return np.asarray(self.s2(C)).reshape(-1, self.n_species)

    def create_1rdm(self, state_idx: int, quantum_part_idx: int, quantum_part_spin_idx: int, C) -> np.ndarray:
        """MO_rdm1 of column state_idx of C as POLYQUANT_DETSET::create_1rdm computes it (rdm1.cpp:4-72)."""
        c = C[:, state_idx] if C.dim() == 2 else C
        return self.rdm1(c, spin=quantum_part_spin_idx, species=quantum_part_idx)

    def release_ham(self):
        check(_lib.load().pq_ci_ham_release(self._h))

    def davidson(self, num_states: int = 1, num_subspace_vec: int = 5, iteration_max: int = 500,
                 convergence_E: float = 1e-6, precision: int = PQ_FP64, energy_shift: float = 0.0,
                 max_subspace: int = 0, return_vectors: bool = False, verbose: bool = False):
        torch = _torch()
        p = _lib.PQDavidsonParams(num_states, num_subspace_vec, max_subspace, iteration_max, convergence_E, precision,
                                  energy_shift, 1 if verbose else 0)
        e = np.zeros(num_states, dtype=np.float64)
        rep = _lib.PQDavidsonReport()
        vecs = None
        vptr = None
        if return_vectors:
            vecs = torch.empty((num_states, self.N_dets), dtype=torch.float64, device="cuda")
            vptr = ctypes.c_void_p(vecs.data_ptr())
        st = _lib.load().pq_ci_davidson(self._h, ctypes.byref(p), e.ctypes.data, vptr, ctypes.byref(rep))
        check(st, "pq_ci_davidson")
        info = dict(iterations=rep.iterations, converged=bool(rep.converged), max_residual=rep.max_residual,
                    sigma_calls_fp64=rep.sigma_calls_fp64, sigma_calls_fp32=rep.sigma_calls_fp32,
                    seconds=rep.seconds, sigma_seconds=rep.sigma_seconds)
        if return_vectors:
            return e, vecs.t(), info
        return e, info
