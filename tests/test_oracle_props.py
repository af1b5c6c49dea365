"""The oracle's <S^2> and 1-RDM (evaluate_s2, src/ci/detset/s2.cpp:4-123; create_1rdm,
src/ci/detset/rdm1.cpp:4-72) against an independent numpy restatement of the same formulas and
against the spin and trace properties of exact eigenvectors."""
import numpy as np
import pytest

import oracle as O
from cases import h2o_problem, synthetic_ep, synthetic_fci


def phase(m, h, p):
    lo, hi = min(h, p), max(h, p)
    return -1.0 if bin(m & (((1 << hi) - 1) ^ ((1 << (lo + 1)) - 1))).count("1") % 2 else 1.0


def masks(d, sp):
    return [int(w[-1]) if np.ndim(w) else int(w) for w in d.strings(0, sp)]


def singles(masks_list):
    out = {}
    for i, m in enumerate(masks_list):
        out[i] = [(j, n) for j, n in enumerate(masks_list) if bin(m ^ n).count("1") == 2]
    return out


def s2_numpy(d, C):
    A, B = masks(d, 0), masks(d, 1)
    u = d.unfold()
    index = {(int(a), int(b)): k for k, (a, b) in enumerate(u)}
    sa = singles(A)
    res = np.zeros(C.shape[1])
    for I, (ia, ib) in enumerate(u):
        am, bm = A[ia], B[ib]
        op = am ^ bm
        n_open, n_a = bin(op).count("1"), bin(op & am).count("1")
        sz = n_a - 0.5 * n_open
        res += C[I] ** 2 * (n_a + sz * (sz - 1.0))
        for ja, jam in sa[ia]:
            ha = (am & ~jam).bit_length() - 1
            pa = (jam & ~am).bit_length() - 1
            if not (bm >> pa) & 1 or (bm >> ha) & 1:
                continue
            jbm = bm ^ (1 << pa) ^ (1 << ha)
            if jbm not in B:
                continue
            J = index.get((ja, B.index(jbm)))
            if J is None:
                continue
            ph = phase(am, ha, pa) * phase(bm, pa, ha)
            res -= ph * C[I] * C[J]
    return res


def rdm1_numpy(d, c, spin, n):
    S = masks(d, spin)
    u = d.unfold()
    index = {(int(a), int(b)): k for k, (a, b) in enumerate(u)}
    ss = singles(S)
    R = np.zeros((n, n))
    for I, key in enumerate(u):
        key = [int(x) for x in key]
        m = S[key[spin]]
        for o in range(n):
            if (m >> o) & 1:
                R[o, o] += c[I] ** 2
        for js, jm in ss[key[spin]]:
            kk = list(key)
            kk[spin] = js
            J = index.get(tuple(kk))
            if J is None or J > I:
                continue
            k = (m & ~jm).bit_length() - 1
            l = (jm & ~m).bit_length() - 1
            v = phase(m, k, l) * c[I] * c[J]
            R[k, l] += v
            R[l, k] += v
    return R


# ---- two species (electron + positron product space) -----------------------
def s2_numpy_two(d, C, sp):
    S = [[[int(w[-1]) for w in d.strings(s, x)] for x in (0, 1)] for s in (0, 1)]
    u = [tuple(int(v) for v in row) for row in d.unfold()]
    index = {key: k for k, key in enumerate(u)}
    res = np.zeros(C.shape[1])
    for I, key in enumerate(u):
        am, bm = S[sp][0][key[2 * sp]], S[sp][1][key[2 * sp + 1]]
        op = am ^ bm
        n_open, n_a = bin(op).count("1"), bin(op & am).count("1")
        sz = n_a - 0.5 * n_open
        res += C[I] ** 2 * (n_a + sz * (sz - 1.0))
        for ja, jam in enumerate(S[sp][0]):
            if bin(am ^ jam).count("1") != 2:
                continue
            ha = (am & ~jam).bit_length() - 1
            pa = (jam & ~am).bit_length() - 1
            if not (bm >> pa) & 1 or (bm >> ha) & 1:
                continue
            jbm = bm ^ (1 << pa) ^ (1 << ha)
            if jbm not in S[sp][1]:
                continue
            kk = list(key)
            kk[2 * sp], kk[2 * sp + 1] = ja, S[sp][1].index(jbm)
            J = index.get(tuple(kk))
            if J is None:
                continue
            res -= phase(am, ha, pa) * phase(bm, pa, ha) * C[I] * C[J]
    return res


def rdm1_numpy_two(d, c, sp, spin, n):
    S = [int(w[-1]) for w in d.strings(sp, spin)]
    u = [tuple(int(v) for v in row) for row in d.unfold()]
    index = {key: k for k, key in enumerate(u)}
    R = np.zeros((n, n))
    slot = 2 * sp + spin
    for I, key in enumerate(u):
        m = S[key[slot]]
        for o in range(n):
            if (m >> o) & 1:
                R[o, o] += c[I] ** 2
        for js, jm in enumerate(S):
            if bin(m ^ jm).count("1") != 2:
                continue
            kk = list(key)
            kk[slot] = js
            J = index.get(tuple(kk))
            if J is None or J > I:
                continue
            k = (m & ~jm).bit_length() - 1
            l = (jm & ~m).bit_length() - 1
            v = phase(m, k, l) * c[I] * c[J]
            R[k, l] += v
            R[l, k] += v
    return R


@pytest.mark.parametrize("which", ["h2o_cisd", "fci_6o_3a2b", "fci_7o_3a3b"])
def test_one_species(which, h2o):
    p = {"h2o_cisd": lambda: h2o_problem(h2o("library"), [2, 2, 2]),
         "fci_6o_3a2b": lambda: synthetic_fci(6, 3, 2, seed=2),
         "fci_7o_3a3b": lambda: synthetic_fci(7, 3, 3, seed=3)}[which]()
    d = O.Detset(p)
    w, V = np.linalg.eigh(d.dense_ham())
    X = V[:, :4]
    s2 = d.evaluate_s2(X)[:, 0]
    assert np.abs(s2 - s2_numpy(d, X)).max() < 1e-11
    S = np.sqrt(s2 + 0.25) - 0.5
    assert np.abs(S - np.round(2 * S) / 2).max() < 1e-6
    Y = np.random.default_rng(1).standard_normal((d.n_dets, 3))
    assert np.abs(d.evaluate_s2(Y)[:, 0] - s2_numpy(d, Y)).max() < 1e-9 * d.n_dets
    c = V[:, 0]
    for spin, ne in ((0, p.n_alpha[0]), (1, p.n_beta[0])):
        R = d.create_1rdm(c, 0, spin)
        assert np.abs(R - rdm1_numpy(d, c, spin, p.n_orb[0])).max() < 1e-13
        assert abs(np.trace(R) - ne) < 1e-10
        ev = np.linalg.eigvalsh(R)
        assert ev.min() > -1e-10 and ev.max() < 1 + 1e-10


@pytest.mark.parametrize("args", [(5, 2, 2, 4, 1, 1, 3), (6, 2, 1, 5, 1, 0, 4)])
def test_two_species(args):
    ne, ea, eb, npo, pa, pb, seed = args
    p = synthetic_ep(ne, ea, eb, npo, pa, pb, seed=seed)
    d = O.Detset(p)
    w, V = np.linalg.eigh(d.dense_ham())
    X = V[:, :3]
    s2 = d.evaluate_s2(X)
    for sp in (0, 1):
        assert np.abs(s2[:, sp] - s2_numpy_two(d, X, sp)).max() < 1e-11
    c = V[:, 0]
    for sp, nel in ((0, (ea, eb)), (1, (pa, pb))):
        for spin in (0, 1):
            R = d.create_1rdm(c, sp, spin)
            assert np.abs(R - rdm1_numpy_two(d, c, sp, spin, p.n_orb[sp])).max() < 1e-13
            assert abs(np.trace(R) - nel[spin]) < 1e-10
