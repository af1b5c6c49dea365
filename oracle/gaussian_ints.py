"""Small Gaussian-integral code for the H2O/STO-3G case -- TEST INFRASTRUCTURE ONLY.

The reference obtains AO integrals from libint2 (integral.cpp:700-1173), which is
not available here.  This module restates the published McMurchie-Davidson
scheme (Hermite expansion coefficients E_t^{ij} and Hermite Coulomb integrals
R_{tuv} over the Boys function) for contracted cartesian s/p Gaussians, enough
for the STO-3G water molecule.  Its results are pinned against the reference's
known AO values (tests/unit_tests/integral/integral_test.cpp:26-53).

Conventions follow the reference: coordinates in Angstrom are converted with
bohr_to_angstrom = 0.529177210903 (molecule.hpp:111); basis functions are
grouped by element in alphabetical order of the element symbol, because the
reference keys its classical particles by symbol in a std::map
(molecule.cpp:265); within an element, atoms follow input order.
"""
from __future__ import annotations

import functools
import itertools
import math

import numpy as np
from scipy.special import gammainc, gamma

BOHR_TO_ANGSTROM = 0.529177210903

# STO-3G (public basis-set data).  Three variants, matching the reference's
# inputs: "file" = the digits of tests/data/h2o_sto3gfile/{H,O}_basis.g94,
# "library" = the 8-digit EMSL values of libint's bundled sto-3g set, and
# "alls" = the file basis with oxygen's SP shell split into three s shells
# (O_basis_sto3galls.g94).
_H_FILE = [("s", [3.425250914, 0.6239137298, 0.1688554040], [0.1543289673, 0.5353281423, 0.4446345422])]
_O_1S_FILE = ("s", [130.7093214, 23.80886605, 6.443608313], [0.1543289673, 0.5353281423, 0.4446345422])
_O_SP_EXP = [5.033151319, 1.169596125, 0.3803889600]
BASES = {
    "file": {
        "H": _H_FILE,
        "O": [_O_1S_FILE, ("s", _O_SP_EXP, [-0.09996722919, 0.3995128261, 0.7001154689]),
              ("p", _O_SP_EXP, [0.1559162750, 0.6076837186, 0.3919573931])],
    },
    "library": {
        "H": [("s", [3.42525091, 0.62391373, 0.16885540], [0.15432897, 0.53532814, 0.44463454])],
        "O": [("s", [130.7093200, 23.8088610, 6.4436083], [0.15432897, 0.53532814, 0.44463454]),
              ("s", [5.0331513, 1.1695961, 0.3803890], [-0.09996723, 0.39951283, 0.70011547]),
              ("p", [5.0331513, 1.1695961, 0.3803890], [0.15591627, 0.60768372, 0.39195739])],
    },
    "alls": {
        "H": _H_FILE,
        "O": [_O_1S_FILE, ("s", _O_SP_EXP, [-0.09996722919, 0.3995128261, 0.7001154689]),
              ("s", _O_SP_EXP, [0.1559162750, 0.6076837186, 0.3919573931])],
    },
}
# "pure": true in the reference inputs -> libint solid-harmonic p order m=-1,0,+1 = (y, z, x)
P_ORDER_PURE = [(0, 1, 0), (0, 0, 1), (1, 0, 0)]
Z = {"H": 1.0, "Li": 3.0, "O": 8.0}


def boys(n: int, T: np.ndarray) -> np.ndarray:
    T = np.asarray(T, dtype=np.float64)
    out = np.empty_like(T)
    small = T < 1e-10
    out[small] = 1.0 / (2 * n + 1) - T[small] / (2 * n + 3)
    Ts = T[~small]
    out[~small] = gamma(n + 0.5) * gammainc(n + 0.5, Ts) / (2.0 * Ts ** (n + 0.5))
    return out


def _E(i, j, t, Qx, a, b):
    """Hermite expansion coefficient E_t^{ij} (McMurchie-Davidson recursion)."""
    p = a + b
    q = a * b / p
    if t < 0 or t > i + j:
        return 0.0
    if i == j == t == 0:
        return math.exp(-q * Qx * Qx)
    if j == 0:
        return (1 / (2 * p)) * _E(i - 1, j, t - 1, Qx, a, b) - (q * Qx / a) * _E(i - 1, j, t, Qx, a, b) + \
            (t + 1) * _E(i - 1, j, t + 1, Qx, a, b)
    return (1 / (2 * p)) * _E(i, j - 1, t - 1, Qx, a, b) + (q * Qx / b) * _E(i, j - 1, t, Qx, a, b) + \
        (t + 1) * _E(i, j - 1, t + 1, Qx, a, b)


def _R(t, u, v, n, p, PCx, PCy, PCz, RPC):
    T = p * RPC * RPC
    val = 0.0
    if t == u == v == 0:
        val += (-2 * p) ** n * float(boys(n, np.array([T]))[0])
    elif t == u == 0:
        if v > 1:
            val += (v - 1) * _R(t, u, v - 2, n + 1, p, PCx, PCy, PCz, RPC)
        val += PCz * _R(t, u, v - 1, n + 1, p, PCx, PCy, PCz, RPC)
    elif t == 0:
        if u > 1:
            val += (u - 1) * _R(t, u - 2, v, n + 1, p, PCx, PCy, PCz, RPC)
        val += PCy * _R(t, u - 1, v, n + 1, p, PCx, PCy, PCz, RPC)
    else:
        if t > 1:
            val += (t - 1) * _R(t - 2, u, v, n + 1, p, PCx, PCy, PCz, RPC)
        val += PCx * _R(t - 1, u, v, n + 1, p, PCx, PCy, PCz, RPC)
    return val


# The recursions are pure functions of their arguments; memoising them makes
# the contracted integrals over repeated primitive pairs several times faster.
_E = functools.lru_cache(maxsize=1 << 20)(_E)
_R = functools.lru_cache(maxsize=1 << 20)(_R)


class Prim:
    __slots__ = ("a", "lmn", "A", "c")

    def __init__(self, a, lmn, A, c):
        self.a, self.lmn, self.A, self.c = a, lmn, np.asarray(A, float), c


def _dfact(n):
    return 1.0 if n <= 0 else float(np.prod(np.arange(n, 0, -2)))


def _prim_norm(a, lmn):
    l, m, n = lmn
    L = l + m + n
    return (2 * a / math.pi) ** 0.75 * (4 * a) ** (L / 2) / math.sqrt(_dfact(2 * l - 1) * _dfact(2 * m - 1) * _dfact(2 * n - 1))


def _overlap_prim(p1: Prim, p2: Prim):
    a, b = p1.a, p2.a
    s = 1.0
    for k in range(3):
        s *= _E(p1.lmn[k], p2.lmn[k], 0, p1.A[k] - p2.A[k], a, b)
    return s * (math.pi / (a + b)) ** 1.5


def _kinetic_prim(p1: Prim, p2: Prim):
    b = p2.b if hasattr(p2, "b") else p2.a
    l, m, n = p2.lmn

    def S(lmn2):
        return _overlap_prim(p1, Prim(p2.a, lmn2, p2.A, 1.0))

    t0 = b * (2 * (l + m + n) + 3) * S((l, m, n))
    t1 = -2 * b * b * (S((l + 2, m, n)) + S((l, m + 2, n)) + S((l, m, n + 2)))
    t2 = -0.5 * (l * (l - 1) * S((l - 2, m, n)) + m * (m - 1) * S((l, m - 2, n)) + n * (n - 1) * S((l, m, n - 2)))
    return t0 + t1 + t2


def _nuclear_prim(p1: Prim, p2: Prim, C):
    a, b = p1.a, p2.a
    p = a + b
    P = (a * p1.A + b * p2.A) / p
    PC = P - C
    RPC = float(np.linalg.norm(PC))
    l1, m1, n1 = p1.lmn
    l2, m2, n2 = p2.lmn
    val = 0.0
    for t in range(l1 + l2 + 1):
        Et = _E(l1, l2, t, p1.A[0] - p2.A[0], a, b)
        for u in range(m1 + m2 + 1):
            Eu = _E(m1, m2, u, p1.A[1] - p2.A[1], a, b)
            for v in range(n1 + n2 + 1):
                Ev = _E(n1, n2, v, p1.A[2] - p2.A[2], a, b)
                val += Et * Eu * Ev * _R(t, u, v, 0, p, PC[0], PC[1], PC[2], RPC)
    return val * 2 * math.pi / p


def _eri_prim(pa: Prim, pb: Prim, pc: Prim, pd: Prim):
    a, b, c, d = pa.a, pb.a, pc.a, pd.a
    p, q = a + b, c + d
    alpha = p * q / (p + q)
    P = (a * pa.A + b * pb.A) / p
    Q = (c * pc.A + d * pd.A) / q
    PQ = P - Q
    RPQ = float(np.linalg.norm(PQ))
    l1, m1, n1 = pa.lmn
    l2, m2, n2 = pb.lmn
    l3, m3, n3 = pc.lmn
    l4, m4, n4 = pd.lmn
    val = 0.0
    for t in range(l1 + l2 + 1):
        E1 = _E(l1, l2, t, pa.A[0] - pb.A[0], a, b)
        for u in range(m1 + m2 + 1):
            E2 = _E(m1, m2, u, pa.A[1] - pb.A[1], a, b)
            for v in range(n1 + n2 + 1):
                E3 = _E(n1, n2, v, pa.A[2] - pb.A[2], a, b)
                for tau in range(l3 + l4 + 1):
                    E4 = _E(l3, l4, tau, pc.A[0] - pd.A[0], c, d)
                    for nu in range(m3 + m4 + 1):
                        E5 = _E(m3, m4, nu, pc.A[1] - pd.A[1], c, d)
                        for phi in range(n3 + n4 + 1):
                            E6 = _E(n3, n4, phi, pc.A[2] - pd.A[2], c, d)
                            val += E1 * E2 * E3 * E4 * E5 * E6 * (-1) ** (tau + nu + phi) * \
                                _R(t + tau, u + nu, v + phi, 0, alpha, PQ[0], PQ[1], PQ[2], RPQ)
    return val * 2 * math.pi ** 2.5 / (p * q * math.sqrt(p + q))


class Molecule:
    """Atoms (symbol, position in bohr) ordered like the reference's AO list."""

    def __init__(self, symbols, geometry_angstrom, basis="file"):
        """``basis``: a name of BASES, or a table {symbol: [(kind, exponents, coefficients), ...]}."""
        table = BASES[basis] if isinstance(basis, str) else basis
        geo = np.asarray(geometry_angstrom, float).reshape(-1, 3) / BOHR_TO_ANGSTROM
        atoms = list(zip(symbols, geo))
        order = sorted(range(len(atoms)), key=lambda k: (atoms[k][0], k))
        self.atoms = [atoms[k] for k in order]
        self.basis = []  # list of contracted functions: list[Prim]
        for sym, pos in self.atoms:
            for kind, exps, coefs in table[sym]:
                lmns = [(0, 0, 0)] if kind == "s" else P_ORDER_PURE
                for lmn in lmns:
                    prims = [Prim(a, lmn, pos, c * _prim_norm(a, lmn)) for a, c in zip(exps, coefs)]
                    norm = 0.0
                    for p1 in prims:
                        for p2 in prims:
                            norm += p1.c * p2.c * _overlap_prim(p1, p2)
                    for p1 in prims:
                        p1.c /= math.sqrt(norm)
                    self.basis.append(prims)

    @property
    def nbf(self):
        return len(self.basis)

    def e_nuc(self) -> float:
        e = 0.0
        for (s1, A), (s2, B) in itertools.combinations(self.atoms, 2):
            e += Z[s1] * Z[s2] / float(np.linalg.norm(A - B))
        return e

    def n_electrons(self) -> int:
        return int(sum(Z[s] for s, _ in self.atoms))

    def one_body(self, nuclear_charges=None):
        """(S, T, V); V attracts to every atom with charge Z[symbol], or with ``nuclear_charges[symbol]`` when
        given (0 for a ghost centre, e.g. a nucleus treated as a quantum particle)."""
        zc = Z if nuclear_charges is None else nuclear_charges
        n = self.nbf
        S = np.zeros((n, n))
        T = np.zeros((n, n))
        V = np.zeros((n, n))
        for i in range(n):
            for j in range(i + 1):
                s = t = v = 0.0
                for p1 in self.basis[i]:
                    for p2 in self.basis[j]:
                        cc = p1.c * p2.c
                        s += cc * _overlap_prim(p1, p2)
                        t += cc * _kinetic_prim(p1, p2)
                        for sym, C in self.atoms:
                            if zc[sym] != 0.0:
                                v -= cc * zc[sym] * _nuclear_prim(p1, p2, C)
                S[i, j] = S[j, i] = s
                T[i, j] = T[j, i] = t
                V[i, j] = V[j, i] = v
        return S, T, V

    def eri_with(self, other: "Molecule") -> np.ndarray:
        """(ij|kl) with i, j over this basis and k, l over ``other``'s (e.g. electron | positron)."""
        return eri_cross(self.basis, other.basis)

    def eri(self) -> np.ndarray:
        n = self.nbf
        out = np.zeros((n, n, n, n))
        for i, j, k, l in itertools.product(range(n), repeat=4):
            ij = i * (i + 1) // 2 + j
            kl = k * (k + 1) // 2 + l
            if j > i or l > k or kl > ij:
                continue
            v = 0.0
            for pa in self.basis[i]:
                for pb in self.basis[j]:
                    for pc in self.basis[k]:
                        for pd in self.basis[l]:
                            v += pa.c * pb.c * pc.c * pd.c * _eri_prim(pa, pb, pc, pd)
            for (a, b, c, d) in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                                 (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)):
                out[a, b, c, d] = v
        return out


def _contracted_eri(fa, fb, fc, fd) -> float:
    v = 0.0
    for pa in fa:
        for pb in fb:
            for pc in fc:
                for pd in fd:
                    v += pa.c * pb.c * pc.c * pd.c * _eri_prim(pa, pb, pc, pd)
    return v


def eri_cross(basis_a, basis_b) -> np.ndarray:
    """Coulomb integrals (ij|kl) between two basis sets, i, j in ``basis_a`` and k, l in ``basis_b``."""
    na, nb = len(basis_a), len(basis_b)
    out = np.zeros((na, na, nb, nb))
    for i in range(na):
        for j in range(i + 1):
            for k in range(nb):
                for l in range(k + 1):
                    v = _contracted_eri(basis_a[i], basis_a[j], basis_b[k], basis_b[l])
                    out[i, j, k, l] = out[j, i, k, l] = out[i, j, l, k] = out[j, i, l, k] = v
    return out


def epscf(species, cross, e_nuc=0.0, conv=1e-12, max_iter=500, cross_repeat_unrestricted=False):
    """Multicomponent Hartree-Fock restating the reference's POLYQUANT_EPSCF fixed point
    (src/scf/epscf.cpp): per species s and spin block,
        F = H_core + J_ss(D_total,s) - K_ss(D_spin) + sum_t q_s q_t J_st(D_total,t)
    with H_core = T / mass - q V (form_H_core, epscf.cpp:5-22), same-species Coulomb and exchange and
    cross-species Coulomb only (form_fock_helper_single_fock_matrix, epscf.cpp:117-273; the density of a
    restricted species with more than one particle is doubled for Coulomb, directscf_get_density_coulomb,
    :82-103), aufbau occupations, and the energies of calculate_E_elec (:519-577).  With
    ``cross_repeat_unrestricted`` the cross-species Coulomb term of a partner species with two spin blocks is
    added once per block, as form_fock_helper (:275-307) does when it loops over the partner's spin blocks with
    the partner's total density each time (so twice); the reference's quantum-nucleus SCF values carry this
    double count.  Converged directly with
    DIIS on F D S - S D F; the reference's staged start (species first independent, then coupled) reaches the
    same fixed point for the ground states used here.

    species: [dict(S, H, eri, n_alpha, n_beta, restricted, charge)], cross: {(0, 1): (ij|kl) with ij of
    species 0 and kl of species 1}.  Returns (E_total, [dict(C, eps, D, F, E) per species]) where C, eps, D
    and F are lists over spin blocks (one block for a restricted species or a single particle)."""
    ns = len(species)
    X = []
    for sp in species:
        w, U = np.linalg.eigh(sp["S"])
        X.append(U @ np.diag(w ** -0.5) @ U.T)
    nblk = [1 if (sp["restricted"] or sp["n_alpha"] + sp["n_beta"] == 1) else 2 for sp in species]
    nocc = [[sp["n_alpha"], sp["n_beta"]][:nblk[k]] for k, sp in enumerate(species)]

    def diag(F, k):
        e, Cp = np.linalg.eigh(X[k].T @ F @ X[k])
        return e, X[k] @ Cp

    C = [[diag(species[k]["H"], k)[1] for _ in range(nblk[k])] for k in range(ns)]
    eps = [[None] * nblk[k] for k in range(ns)]

    def densities(C):
        return [[C[k][b][:, :nocc[k][b]] @ C[k][b][:, :nocc[k][b]].T for b in range(nblk[k])] for k in range(ns)]

    def total(D, k):
        sp = species[k]
        if nblk[k] == 2:
            return D[k][0] + D[k][1]
        return 2.0 * D[k][0] if sp["n_alpha"] + sp["n_beta"] > 1 else D[k][0]

    def fock(D):
        F = []
        for k, sp in enumerate(species):
            Jk = np.einsum("pqrs,rs->pq", sp["eri"], total(D, k), optimize=True)
            G = sp["H"] + Jk
            for t in range(ns):
                if t == k:
                    continue
                qq = sp["charge"] * species[t]["charge"]
                if cross_repeat_unrestricted and nblk[t] == 2:
                    qq *= 2.0  # the reference adds the partner's Coulomb term once per spin block
                if (k, t) in cross:
                    G = G + qq * np.einsum("pqrs,rs->pq", cross[(k, t)], total(D, t), optimize=True)
                else:
                    G = G + qq * np.einsum("rspq,rs->pq", cross[(t, k)], total(D, t), optimize=True)
            F.append([G - np.einsum("prqs,rs->pq", sp["eri"], D[k][b], optimize=True) for b in range(nblk[k])])
        return F

    def energies(D, F):
        E = []
        for k, sp in enumerate(species):
            H = sp["H"]
            if sp["n_alpha"] + sp["n_beta"] == 1:
                E.append(0.5 * np.sum(D[k][0] * (H + F[k][0])))
            elif nblk[k] == 2:
                E.append(0.5 * np.sum((D[k][0] + D[k][1]) * H + D[k][0] * F[k][0] + D[k][1] * F[k][1]))
            else:
                E.append(np.sum(D[k][0] * (H + F[k][0])))
        return E

    hist_F, hist_e = [], []
    E_old = None
    for _ in range(max_iter):
        D = densities(C)
        F = fock(D)
        E = energies(D, F)
        errs = [F[k][b] @ D[k][b] @ species[k]["S"] - species[k]["S"] @ D[k][b] @ F[k][b]
                for k in range(ns) for b in range(nblk[k])]
        err = max(float(np.abs(e).max()) for e in errs)
        Et = sum(E) + e_nuc
        if E_old is not None and abs(Et - E_old) < conv and err < 1e-10:
            break
        E_old = Et
        hist_F.append(F)
        hist_e.append(np.concatenate([e.ravel() for e in errs]))
        hist_F, hist_e = hist_F[-10:], hist_e[-10:]
        m = len(hist_F)
        Fx = F
        if m > 1:
            B = -np.ones((m + 1, m + 1))
            B[m, m] = 0.0
            for a in range(m):
                for b in range(m):
                    B[a, b] = hist_e[a] @ hist_e[b]
            rhs = np.zeros(m + 1)
            rhs[m] = -1.0
            coef = np.linalg.solve(B, rhs)[:m]
            Fx = [[sum(c * hf[k][b] for c, hf in zip(coef, hist_F)) for b in range(nblk[k])] for k in range(ns)]
        for k in range(ns):
            for b in range(nblk[k]):
                eps[k][b], C[k][b] = diag(Fx[k][b], k)
    D = densities(C)
    F = fock(D)
    E = energies(D, F)
    out = [dict(C=C[k], eps=[diag(F[k][b], k)[0] for b in range(nblk[k])], D=D[k], F=F[k], E=E[k])
           for k in range(ns)]
    return sum(E) + e_nuc, out


def rhf(S, hcore, eri, n_occ, e_nuc, conv=1e-12, max_iter=200):
    """Restricted Hartree-Fock with DIIS; returns (E_total, C, orbital energies)."""
    s, U = np.linalg.eigh(S)
    X = U @ np.diag(s ** -0.5) @ U.T
    e, Cp = np.linalg.eigh(X.T @ hcore @ X)
    C = X @ Cp
    D = 2 * C[:, :n_occ] @ C[:, :n_occ].T
    E_old = 0.0
    focks, errs = [], []
    for _ in range(max_iter):
        J = np.einsum("pqrs,rs->pq", eri, D)
        K = np.einsum("prqs,rs->pq", eri, D)
        F = hcore + J - 0.5 * K
        err = F @ D @ S - S @ D @ F
        focks.append(F)
        errs.append(err)
        focks, errs = focks[-8:], errs[-8:]
        if len(focks) > 1:
            m = len(focks)
            B = -np.ones((m + 1, m + 1))
            B[m, m] = 0.0
            for a in range(m):
                for b in range(m):
                    B[a, b] = np.sum(errs[a] * errs[b])
            rhs = np.zeros(m + 1)
            rhs[m] = -1.0
            coef = np.linalg.solve(B, rhs)[:m]
            F = sum(c * f for c, f in zip(coef, focks))
        e, Cp = np.linalg.eigh(X.T @ F @ X)
        C = X @ Cp
        D = 2 * C[:, :n_occ] @ C[:, :n_occ].T
        E = 0.5 * np.sum(D * (hcore + F)) + e_nuc
        if abs(E - E_old) < conv and np.max(np.abs(err)) < 1e-8:
            break
        E_old = E
    # final energy from an un-extrapolated Fock build
    J = np.einsum("pqrs,rs->pq", eri, D)
    K = np.einsum("prqs,rs->pq", eri, D)
    F = hcore + J - 0.5 * K
    E = 0.5 * np.sum(D * (hcore + F)) + e_nuc
    return E, C, e


# H2O geometry of the reference's sto-3g inputs (tests/data/h2o_sto3gfile/h2o.json)
H2O_SYMBOLS = ["H", "H", "O"]
H2O_GEOMETRY = [0.7569685, 0.0, -0.5858752, -0.7569685, 0.0, -0.5858752, 0.0, 0.0, 0.0]


def h2o_sto3g(basis: str = "file"):
    """AO integrals, nuclear repulsion and RHF solution of H2O/STO-3G."""
    mol = Molecule(H2O_SYMBOLS, H2O_GEOMETRY, basis)
    S, T, V = mol.one_body()
    eri = mol.eri()
    E, C, eps = rhf(S, T + V, eri, mol.n_electrons() // 2, mol.e_nuc())
    return dict(S=S, T=T, V=V, eri=eri, e_nuc=mol.e_nuc(), E_rhf=E, C=C, eps=eps)
