"""Host model of the FP32 sigma's tensor-core arithmetic (the FP16 hi/lo split of ci_sigma32_ss.cu and
ci_sigma32_tc.cu): both operands scaled by powers of two into [2^14, 2^15), split x = hi + lo with hi, lo in
FP16, and the product formed as hi*hi + hi*lo + lo*hi with FP32 accumulation.  On the same-spin doubles of a
small full-CI space (the dense string x string matrix the GEMMs use) and on random vectors, the model stays
within the 2e-5 relative sigma tolerance of the GPU tests and close to plain FP32 arithmetic, and the scaling
keeps that accuracy for vectors of very small and very large magnitude."""
import itertools

import numpy as np


def _scale(x):
    """Power of two 2^e with max|x| * 2^e in [2^14, 2^15) (1 for x == 0), as fp16_scale does."""
    m = float(np.abs(x).max())
    if m == 0.0 or not np.isfinite(m):
        return 1.0
    _, e = np.frexp(m)
    return float(np.ldexp(1.0, 15 - int(e)))


def _split(x):
    hi = x.astype(np.float16)
    lo = (x - hi.astype(np.float32)).astype(np.float16)
    return hi, lo


def split_product(D, X):
    """D (m x k) times X (k x n) in the split arithmetic; every FP16 x FP16 product is exact in FP32."""
    sd, sx = _scale(D), _scale(X)
    dh, dl = _split((D * sd).astype(np.float32))
    xh, xl = _split((X * sx).astype(np.float32))
    f32 = lambda a: a.astype(np.float32)
    acc = f32(dh) @ f32(xh) + f32(dh) @ f32(xl) + f32(dl) @ f32(xh)
    return acc.astype(np.float64) / sd / sx


def _same_spin_doubles(n, ne, seed):
    """Dense same-spin doubles matrix over the strings of ne electrons in n orbitals: antisymmetrised random
    two-electron integrals on the pairs of strings that differ by two orbitals (the structure, not the values,
    of the matrix the GEMMs multiply)."""
    S = [sum(1 << i for i in c) for c in itertools.combinations(range(n), ne)]
    rng = np.random.default_rng(seed)
    D = np.zeros((len(S), len(S)))
    for i, a in enumerate(S):
        for j, b in enumerate(S):
            if i < j and bin(a ^ b).count("1") == 4:
                D[i, j] = D[j, i] = rng.standard_normal() * 0.3
    return D


def test_split_product_meets_the_fp32_sigma_tolerance():
    D = _same_spin_doubles(9, 4, seed=1)  # 126 strings, 60 doubles per string
    rng = np.random.default_rng(2)
    X = rng.standard_normal((D.shape[0], 4 * 40))
    exact = D @ X
    scale = np.abs(exact).max()
    err_split = np.abs(split_product(D, X) - exact).max() / scale
    err_fp32 = np.abs((D.astype(np.float32) @ X.astype(np.float32)).astype(np.float64) - exact).max() / scale
    assert err_split < 2e-5
    assert err_split < 10 * max(err_fp32, 1e-7)


def test_power_of_two_scaling_keeps_relative_accuracy():
    D = _same_spin_doubles(8, 3, seed=3)
    rng = np.random.default_rng(4)
    for f in (1e-30, 1.0, 1e20):
        X = f * rng.standard_normal((D.shape[0], 16))
        exact = D @ X
        err = np.abs(split_product(D, X) - exact).max() / np.abs(exact).max()
        assert err < 2e-5, (f, err)


def test_scale_brings_the_largest_value_into_the_top_binade():
    for m in (1e-30, 3.7e-5, 1.0, 2.0, 6.5e4, 1e20):
        s = _scale(np.array([m, -m / 3]))
        assert 2.0 ** 14 <= m * s < 2.0 ** 15
        assert np.log2(s) == int(np.log2(s))  # a power of two: exact in FP32, no rounding of the data
