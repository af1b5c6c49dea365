"""CPU oracle for the polyquant CI path -- TEST INFRASTRUCTURE ONLY.

Python access (ctypes) to the plain-C restatement in ``pq_oracle.c`` of the
reference's determinant, Slater-Condon and sigma algorithms
(polyquant ``src/ci/detset/*.cpp``), plus numpy restatements of the integral
transform (``src/integral/integral.cpp:166-516``).  Only the test-suite, the
smoke check and the CPU-baseline leg of ``bench.py`` import this module; the
product library never calls it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libpq_oracle.so")
_lib = None


_REFALG_PATH = os.path.join(_BUILD, "libpq_refalg.so")
_refalg = None


def build(force: bool = False) -> str:
    """Compile the C oracle into ``oracle/_build/libpq_oracle.so`` (gcc + OpenMP)."""
    src = os.path.join(_HERE, "pq_oracle.c")
    hdr = os.path.join(_HERE, "pq_oracle.h")
    if (force or not os.path.exists(_LIB_PATH)
            or os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(src), os.path.getmtime(hdr))):
        os.makedirs(_BUILD, exist_ok=True)
        tmp = _LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def build_refalg(force: bool = False) -> str:
    """Compile the reference-faithful sigma restatement (ref_restated.cpp) into ``oracle/_build/libpq_refalg.so``
    (g++ + OpenMP, linked against the oracle); built on first use only."""
    build()
    ref = os.path.join(_HERE, "ref_restated.cpp")
    if (force or not os.path.exists(_REFALG_PATH)
            or os.path.getmtime(_REFALG_PATH) < max(os.path.getmtime(ref), os.path.getmtime(_LIB_PATH))):
        tmp = _REFALG_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-I", _HERE, "-o", tmp,
                               ref, "-L", _BUILD, "-lpq_oracle", "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, _REFALG_PATH)
    return _REFALG_PATH


class OrcDesc(ctypes.Structure):
    _fields_ = [
        ("n_species", ctypes.c_int32),
        ("n_orb", ctypes.c_int32 * 2),
        ("n_alpha", ctypes.c_int32 * 2),
        ("n_beta", ctypes.c_int32 * 2),
        ("restricted", ctypes.c_int32 * 2),
        ("charge", ctypes.c_double * 2),
        ("ex_level", (ctypes.c_int32 * 3) * 2),
        ("max_collective", ctypes.c_int32),
        ("h1", (ctypes.c_void_p * 2) * 2),
        ("eri", ((((ctypes.c_void_p * 2) * 2) * 2) * 2)),
    ]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        L = _lib
        P, I32, I64, D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
        L.orc_detset_create.restype = P
        L.orc_detset_create.argtypes = [ctypes.POINTER(OrcDesc), ctypes.c_int]
        L.orc_detset_destroy.argtypes = [P]
        L.orc_n_words.restype = ctypes.c_int
        L.orc_n_words.argtypes = [P]
        L.orc_n_dets.restype = I64
        L.orc_n_dets.argtypes = [P]
        L.orc_n_strings.restype = I64
        L.orc_n_strings.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_strings.restype = P
        L.orc_strings.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_unfold.restype = P
        L.orc_unfold.argtypes = [P]
        L.orc_lookup.restype = I64
        L.orc_lookup.argtypes = [P, P]
        for f in (L.orc_singles, L.orc_doubles):
            f.restype = I64
            f.argtypes = [P, ctypes.c_int, ctypes.c_int, I64, ctypes.POINTER(ctypes.POINTER(I32))]
        L.orc_diagonal.restype = P
        L.orc_diagonal.argtypes = [P]
        for f in (L.orc_same_part_ham_diag, L.orc_same_part_ham_single, L.orc_same_part_ham_double):
            f.restype = D
            f.argtypes = [P, ctypes.c_int, P, P]
        for f in (L.orc_mixed_part_ham_diag, L.orc_mixed_part_ham_single, L.orc_mixed_part_ham_double):
            f.restype = D
            f.argtypes = [P, ctypes.c_int, ctypes.c_int, P, P]
        L.orc_slater_condon.restype = D
        L.orc_slater_condon.argtypes = [P, I64, I64]
        for f in (L.orc_sigma_singleshot, L.orc_sigma_slow):
            f.argtypes = [P, P, I64, ctypes.c_int, P, I64, ctypes.c_int]
        L.orc_sigma_rows.argtypes = [P, P, I64, ctypes.c_int, P, I64, P, ctypes.c_int]
        L.orc_dense_ham.argtypes = [P, P, ctypes.c_int]
        L.orc_evaluate_s2.argtypes = [P, P, I64, ctypes.c_int, P, ctypes.c_int]
        L.orc_create_1rdm.argtypes = [P, P, ctypes.c_int, ctypes.c_int, P, ctypes.c_int]
        L.orc_single_spin_num_excitation.restype = ctypes.c_int
        L.orc_single_spin_num_excitation.argtypes = [P, P, ctypes.c_int]
        L.orc_get_holes.restype = ctypes.c_int
        L.orc_get_holes.argtypes = [P, P, ctypes.c_int, P]
        L.orc_get_parts.restype = ctypes.c_int
        L.orc_get_parts.argtypes = [P, P, ctypes.c_int, P]
        L.orc_get_phase.restype = D
        L.orc_get_phase.argtypes = [P, P, ctypes.c_int, P, P, ctypes.c_int]
        L.orc_get_occ_virt.restype = ctypes.c_int
        L.orc_get_occ_virt.argtypes = [P, ctypes.c_int, ctypes.c_int, P, P, P, P]
        L.orc_idx2.restype = ctypes.c_int
        L.orc_idx2.argtypes = [ctypes.c_int, ctypes.c_int]
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# --------------------------------------------------------------------------
# bit operations (determinant_operations.cpp)
def _words(v) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v, dtype=np.uint64))


def num_excitation(Di, Dj) -> int:
    a, b = _words(Di), _words(Dj)
    return lib().orc_single_spin_num_excitation(_ptr(a), _ptr(b), len(a))


def get_holes(Di, Dj) -> list:
    a, b = _words(Di), _words(Dj)
    out = np.zeros(64 * len(a), dtype=np.int32)
    n = lib().orc_get_holes(_ptr(a), _ptr(b), len(a), _ptr(out))
    return out[:n].tolist()


def get_parts(Di, Dj) -> list:
    a, b = _words(Di), _words(Dj)
    out = np.zeros(64 * len(a), dtype=np.int32)
    n = lib().orc_get_parts(_ptr(a), _ptr(b), len(a), _ptr(out))
    return out[:n].tolist()


def get_phase(Di, Dj, holes, parts) -> float:
    a, b = _words(Di), _words(Dj)
    h = np.asarray(holes, dtype=np.int32)
    p = np.asarray(parts, dtype=np.int32)
    return lib().orc_get_phase(_ptr(a), _ptr(b), len(a), _ptr(h), _ptr(p), len(h))


def get_occ_virt(D, max_orb: int):
    a = _words(D)
    occ = np.zeros(64 * len(a), dtype=np.int32)
    virt = np.zeros(64 * len(a), dtype=np.int32)
    no = ctypes.c_int(0)
    nv = ctypes.c_int(0)
    lib().orc_get_occ_virt(_ptr(a), len(a), max_orb, _ptr(occ), ctypes.addressof(no), _ptr(virt), ctypes.addressof(nv))
    return occ[: no.value].tolist(), virt[: nv.value].tolist()


def idx2(i: int, j: int) -> int:
    return lib().orc_idx2(i, j)


# --------------------------------------------------------------------------
class CIProblem:
    """One CI problem in the reference's conventions.

    h1[s][spin]: (n_orb x n_orb) MO one-body integrals;
    eri[(a, sa, b, sb)]: (npair_a x npair_b) MO ERIs at [idx2(i,j), idx2(k,l)],
    b >= a (integral.cpp:479-516).  Restricted species carry one spin block.
    """

    def __init__(self, n_orb: Sequence[int], n_alpha: Sequence[int], n_beta: Sequence[int], h1, eri,
                 ex_level: Sequence[Sequence[int]], restricted: Sequence[int] = None, charge: Sequence[float] = None,
                 max_collective: int = 2 ** 31 - 1, e_const: float = 0.0):
        self.n_species = len(n_orb)
        self.n_orb = list(n_orb)
        self.n_alpha = list(n_alpha)
        self.n_beta = list(n_beta)
        self.restricted = list(restricted) if restricted is not None else [1] * self.n_species
        self.charge = list(charge) if charge is not None else [-1.0] * self.n_species
        self.ex_level = [list(e) for e in ex_level]
        self.max_collective = int(max_collective)
        self.e_const = float(e_const)
        self.h1 = [[np.asfortranarray(np.asarray(m, dtype=np.float64)) for m in hs] for hs in h1]
        self.eri = {k: np.asfortranarray(np.asarray(v, dtype=np.float64)) for k, v in eri.items()}

    def spin_blocks(self, s: int) -> int:
        return 1 if self.restricted[s] else 2

    def desc_fields(self):
        """(field values, arrays to keep alive); pointers are host addresses."""
        keep = []
        h1p = [[None, None], [None, None]]
        erip = {}
        for s in range(self.n_species):
            nb = self.spin_blocks(s)
            for sp in range(2):
                m = self.h1[s][sp % nb]
                keep.append(m)
                h1p[s][sp] = m.ctypes.data
        for a in range(self.n_species):
            for sa in range(2):
                for b in range(self.n_species):
                    for sb in range(2):
                        aa, bb, xa, xb = a, b, sa, sb
                        if bb < aa:
                            continue
                        key = (aa, xa % self.spin_blocks(aa), bb, xb % self.spin_blocks(bb))
                        if key not in self.eri:
                            continue
                        m = self.eri[key]
                        keep.append(m)
                        erip[(a, sa, b, sb)] = m.ctypes.data
        return h1p, erip, keep

    def orc_desc(self):
        d = OrcDesc()
        d.n_species = self.n_species
        for s in range(self.n_species):
            d.n_orb[s] = self.n_orb[s]
            d.n_alpha[s] = self.n_alpha[s]
            d.n_beta[s] = self.n_beta[s]
            d.restricted[s] = self.restricted[s]
            d.charge[s] = self.charge[s]
            for t in range(3):
                d.ex_level[s][t] = self.ex_level[s][t]
        d.max_collective = self.max_collective
        h1p, erip, keep = self.desc_fields()
        for s in range(2):
            for sp in range(2):
                d.h1[s][sp] = h1p[s][sp]
        for (a, sa, b, sb), p in erip.items():
            d.eri[a][sa][b][sb] = p
        return d, keep


class Detset:
    """Oracle determinant set (POLYQUANT_DETSET restated)."""

    def __init__(self, prob: CIProblem, check_addressing: bool = True):
        self.prob = prob
        self._desc, self._keep = prob.orc_desc()
        L = lib()
        self._h = L.orc_detset_create(ctypes.byref(self._desc), 1 if check_addressing else 0)
        if not self._h:
            raise ValueError("oracle detset creation failed (excitation level exceeds the virtual orbitals, or an "
                             "integral block is missing)")
        self.n_dets = L.orc_n_dets(self._h)
        self.n_words = L.orc_n_words(self._h)
        self.ntup = 2 * prob.n_species

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_detset_destroy(self._h)
            self._h = None

    def strings(self, s: int, sp: int) -> np.ndarray:
        L = lib()
        n = L.orc_n_strings(self._h, s, sp)
        p = L.orc_strings(self._h, s, sp)
        arr = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint64)), shape=(n * self.n_words,))
        return arr.reshape(n, self.n_words).copy()

    def unfold(self) -> np.ndarray:
        p = lib().orc_unfold(self._h)
        arr = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_int32)), shape=(self.n_dets * self.ntup,))
        return arr.reshape(self.n_dets, self.ntup).copy()

    def lookup(self, tup) -> int:
        t = np.asarray(list(tup) + [0] * (4 - len(tup)), dtype=np.int32)
        return lib().orc_lookup(self._h, _ptr(t))

    def singles(self, s: int, sp: int, I: int) -> np.ndarray:
        ptr = ctypes.POINTER(ctypes.c_int32)()
        n = lib().orc_singles(self._h, s, sp, I, ctypes.byref(ptr))
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy() if n else np.zeros(0, np.int32)

    def doubles(self, s: int, sp: int, I: int) -> np.ndarray:
        ptr = ctypes.POINTER(ctypes.c_int32)()
        n = lib().orc_doubles(self._h, s, sp, I, ctypes.byref(ptr))
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy() if n else np.zeros(0, np.int32)

    def diagonal(self) -> np.ndarray:
        p = lib().orc_diagonal(self._h)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_double)), shape=(self.n_dets,)).copy()

    def _tup(self, t):
        return np.asarray(list(t) + [0] * (4 - len(t)), dtype=np.int32)

    def same_part_ham_diag(self, part, I, J):
        a, b = self._tup(I), self._tup(J)
        return lib().orc_same_part_ham_diag(self._h, part, _ptr(a), _ptr(b))

    def same_part_ham_single(self, part, I, J):
        a, b = self._tup(I), self._tup(J)
        return lib().orc_same_part_ham_single(self._h, part, _ptr(a), _ptr(b))

    def same_part_ham_double(self, part, I, J):
        a, b = self._tup(I), self._tup(J)
        return lib().orc_same_part_ham_double(self._h, part, _ptr(a), _ptr(b))

    def slater_condon(self, i: int, j: int) -> float:
        return lib().orc_slater_condon(self._h, i, j)

    def dense_ham(self, nthreads: int = 0) -> np.ndarray:
        H = np.zeros((self.n_dets, self.n_dets), dtype=np.float64, order="F")
        lib().orc_dense_ham(self._h, _ptr(H), nthreads)
        return H

    def sigma(self, C: np.ndarray, nthreads: int = 0, slow: bool = False) -> np.ndarray:
        C = np.asfortranarray(np.asarray(C, dtype=np.float64).reshape(self.n_dets, -1))
        S = np.zeros_like(C, order="F")
        f = lib().orc_sigma_slow if slow else lib().orc_sigma_singleshot
        f(self._h, _ptr(C), self.n_dets, C.shape[1], _ptr(S), self.n_dets, nthreads)
        return S

    def evaluate_s2(self, C: np.ndarray, nthreads: int = 0) -> np.ndarray:
        """<S^2> of each column of C per species (s2.cpp:4-123): shape (k, n_species)."""
        C = np.asfortranarray(np.asarray(C, dtype=np.float64).reshape(self.n_dets, -1))
        out = np.zeros((C.shape[1], self.prob.n_species), order="F")
        lib().orc_evaluate_s2(self._h, _ptr(C), self.n_dets, C.shape[1], _ptr(out), nthreads)
        return out

    def create_1rdm(self, c: np.ndarray, species: int = 0, spin: int = 0, nthreads: int = 0) -> np.ndarray:
        """One-particle density matrix of one state (rdm1.cpp:4-72): n_orb x n_orb."""
        c = np.ascontiguousarray(np.asarray(c, dtype=np.float64).reshape(-1))
        n = self.prob.n_orb[species]
        out = np.zeros((n, n), order="F")
        lib().orc_create_1rdm(self._h, _ptr(c), species, spin, _ptr(out), nthreads)
        return out

    def sigma_rows(self, C: np.ndarray, rows, nthreads: int = 0) -> np.ndarray:
        C = np.asfortranarray(np.asarray(C, dtype=np.float64).reshape(self.n_dets, -1))
        r = np.ascontiguousarray(np.asarray(rows, dtype=np.int64))
        S = np.zeros((len(r), C.shape[1]), dtype=np.float64, order="F")
        lib().orc_sigma_rows(self._h, _ptr(C), self.n_dets, C.shape[1], _ptr(r), len(r), _ptr(S), nthreads)
        return S


class RefAlgDetset:
    """The reference's sigma builders (one and two species) with its own data structures (hash-map determinant
    index, linear det_idx_unfold, per-thread private sigma, critical merge; ref_restated.cpp), for timing the
    reference algorithm and for checking it against the oracle."""

    def __init__(self, prob: CIProblem):
        global _refalg
        lib()  # the oracle library it links against
        if _refalg is None:
            _refalg = ctypes.CDLL(build_refalg())
            _refalg.refalg_create.restype = ctypes.c_void_p
            _refalg.refalg_create.argtypes = [ctypes.POINTER(OrcDesc)]
            _refalg.refalg_destroy.argtypes = [ctypes.c_void_p]
            _refalg.refalg_n_dets.restype = ctypes.c_int64
            _refalg.refalg_n_dets.argtypes = [ctypes.c_void_p]
            _refalg.refalg_sigma.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                             ctypes.c_void_p, ctypes.c_int64, ctypes.c_int]
        self._desc, self._keep = prob.orc_desc()
        self._h = _refalg.refalg_create(ctypes.byref(self._desc))
        if not self._h:
            raise ValueError("reference restatement: one or two species, with complete integral blocks")
        self.n_dets = _refalg.refalg_n_dets(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            _refalg.refalg_destroy(self._h)
            self._h = None

    def sigma(self, C: np.ndarray, nthreads: int = 0) -> np.ndarray:
        C = np.asfortranarray(np.asarray(C, dtype=np.float64).reshape(self.n_dets, -1))
        S = np.zeros_like(C, order="F")
        _refalg.refalg_sigma(self._h, _ptr(C), self.n_dets, C.shape[1], _ptr(S), self.n_dets, nthreads)
        return S


# --------------------------------------------------------------------------
# integral transform restatements (integral.cpp:166-205, 207-477)
def idx2_array(n: int) -> np.ndarray:
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    return np.where(i > j, i * (i + 1) // 2 + j, j * (j + 1) // 2 + i)


def mo_one_body(C: np.ndarray, hcore_ao: np.ndarray) -> np.ndarray:
    """h_MO = C^T (T - qV) C  (integral.cpp:166-205, frozen core absent)."""
    return C.T @ hcore_ao @ C


def ao2mo_full(eri_ao: np.ndarray, Ca: np.ndarray, Cb: np.ndarray) -> np.ndarray:
    """(ij|kl) = sum C_pi C_qj C_rk C_sl (pq|rs) from a full 4-index AO tensor,
    returned in the reference layout (npair_a x npair_b, idx2 pairs),
    integral.cpp:207-477."""
    t = np.einsum("pqrs,pi->iqrs", eri_ao, Ca, optimize=True)
    t = np.einsum("iqrs,qj->ijrs", t, Ca, optimize=True)
    t = np.einsum("ijrs,rk->ijks", t, Cb, optimize=True)
    t = np.einsum("ijks,sl->ijkl", t, Cb, optimize=True)
    return pack_pairs(t)


def pack_pairs(t: np.ndarray) -> np.ndarray:
    na, nb = t.shape[0], t.shape[2]
    ia, ja = np.tril_indices(na)  # i >= j -> idx2 = i(i+1)/2 + j, row-major tril order
    ib, jb = np.tril_indices(nb)
    return np.ascontiguousarray(t[ia, ja][:, ib, jb])


def unpack_packed8(packed: np.ndarray, n: int) -> np.ndarray:
    """Full (pq|rs) from an 8-fold packed vector at idx2(idx2(p,q), idx2(r,s))."""
    p2 = idx2_array(n)
    npair = n * (n + 1) // 2
    P = p2.reshape(-1)
    full_pairs = np.empty((npair, npair), dtype=packed.dtype)
    a, b = np.meshgrid(np.arange(npair), np.arange(npair), indexing="ij")
    full_pairs[:] = packed[np.where(a > b, a * (a + 1) // 2 + b, b * (b + 1) // 2 + a)]
    return full_pairs[P][:, P].reshape(n, n, n, n)


def ao2mo_rows_factorized(Bp: np.ndarray, C: np.ndarray, rows, block: int = 64) -> np.ndarray:
    """Selected rows of the MO pair matrix for AO integrals given in factorized form
    (mu nu|la si) = sum_L Bp[L, mu nu] Bp[L, la si] (pairs in idx2 order).  The four quarter transforms of
    integral.cpp:207-477 applied to each factor give M_L = C^T B_L C, so
    (ij|kl) = sum_L M_L[ij] M_L[kl]; returned as (len(rows) x npair_mo) at [row, idx2(k, l)], the reference
    layout's rows.  Exact in FP64 up to rounding, at a cost that allows N_AO = 256 on the host."""
    n = C.shape[0]
    n_mo = C.shape[1]
    i, j = np.tril_indices(n)
    im, jm = np.tril_indices(n_mo)
    L = Bp.shape[0]
    M = np.empty((L, len(im)))
    for l0 in range(0, L, block):
        l1 = min(L, l0 + block)
        B = np.zeros((l1 - l0, n, n))
        B[:, i, j] = Bp[l0:l1]
        B[:, j, i] = Bp[l0:l1]
        T = np.matmul(np.matmul(C.T[None], B), C[None])
        M[l0:l1] = T[:, im, jm]
    rows = np.asarray(rows, dtype=np.int64)
    return M[:, rows].T @ M
