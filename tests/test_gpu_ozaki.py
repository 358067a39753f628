"""GPU: the FP64-accurate tensor-core GEMM (exact BF16 slicing, tcgen05)
against cuBLAS FP64 and against exact integer products."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oz(A, B):
    import torch
    from flare_gb300 import _lib
    M, K = A.shape
    N = B.shape[0]
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    dC = torch.full((max(M, 1), max(N, 1)), np.nan, dtype=torch.float64,
                    device="cuda")
    _lib.check(_lib.lib().fgb_oz_dgemm_nt(M, N, K, _lib.ptr(dA), K,
                                          _lib.ptr(dB), K, _lib.ptr(dC),
                                          max(N, 1), _lib.stream_ptr()))
    torch.cuda.synchronize()
    return dC.cpu().numpy()[:M, :N]


@pytest.mark.parametrize("M,N,K", [(128, 48, 32), (300, 130, 680),
                                   (257, 1000, 1000), (5, 3, 17)])
def test_random_fp64_accuracy(M, N, K):
    r = np.random.Generator(np.random.PCG64(M * 7 + N))
    # entries spanning several decades, mixed signs
    A = r.normal(size=(M, K)) * np.exp(r.uniform(-6, 2, size=(M, K)))
    B = r.normal(size=(N, K)) * np.exp(r.uniform(-6, 2, size=(N, K)))
    C = oz(A, B)
    ref = A @ B.T
    bound = np.abs(A).max(1)[:, None] * np.abs(B).sum(1)[None, :] + \
        np.abs(A).sum(1)[:, None] * np.abs(B).max(1)[None, :]
    err = np.abs(C - ref)
    assert np.all(err <= 2e-15 * bound + 1e-300), float((err / bound).max())


def test_integer_products_exact():
    r = np.random.Generator(np.random.PCG64(3))
    A = r.integers(-100, 101, size=(200, 512)).astype(np.float64)
    B = r.integers(-100, 101, size=(100, 512)).astype(np.float64)
    C = oz(A, B)
    exact = (A.astype(np.int64) @ B.astype(np.int64).T).astype(np.float64)
    np.testing.assert_array_equal(C, exact)


def test_worst_case_magnitudes_at_max_k():
    """K at the exact-accumulation limit with every slice at its largest."""
    K = 1472
    A = np.full((130, K), 0.99609375 - 1e-12)
    B = np.full((50, K), -(0.99609375 - 1e-12))
    B[::2] *= -1
    C = oz(A, B)
    ref = A @ B.T
    # no cancellation here: only the slice residuals and the FP64
    # recombination round (the exactness of the FP32 group sums is what
    # this shape checks; a lost bit would show at 1e-7)
    np.testing.assert_allclose(C, ref, rtol=1e-14)


@pytest.mark.parametrize("K", [1473, 3000, 4000])
def test_k_segments(K):
    """K beyond one exact-accumulation segment (1472): the kernel restarts
    the TMEM accumulators per segment and adds the exact group sums in
    64-bit integers, so the bound is unchanged."""
    r = np.random.Generator(np.random.PCG64(K))
    A = r.normal(size=(150, K)) * np.exp(r.uniform(-4, 1, size=(150, K)))
    B = r.normal(size=(70, K)) * np.exp(r.uniform(-4, 1, size=(70, K)))
    C = oz(A, B)
    ref = A @ B.T
    bound = np.abs(A).max(1)[:, None] * np.abs(B).sum(1)[None, :] + \
        np.abs(A).sum(1)[:, None] * np.abs(B).max(1)[None, :]
    err = np.abs(C - ref)
    assert np.all(err <= 2e-15 * bound + 1e-300), float((err / bound).max())


def test_worst_case_magnitudes_two_segments():
    """Every slice at its largest over three segments (2 x 1472 + 56)."""
    K = 3000
    A = np.full((130, K), 0.99609375 - 1e-12)
    B = np.full((50, K), -(0.99609375 - 1e-12))
    B[::2] *= -1
    np.testing.assert_allclose(oz(A, B), A @ B.T, rtol=1e-14)


@pytest.mark.parametrize("sa,sb", [(1e-150, 1e-150), (1e150, 1e-160),
                                   (1e100, 1e100), (2.0 ** -1000, 2.0 ** 60)])
def test_extreme_row_scales(sa, sb):
    """Row scales far from 1: the power-of-two scalings and the integer
    construction of the result doubles (including results near the bottom
    of the normal range) stay FP64-accurate."""
    r = np.random.Generator(np.random.PCG64(11))
    A = r.normal(size=(140, 96)) * sa
    B = r.normal(size=(60, 96)) * sb
    C = oz(A, B)
    ref = A @ B.T
    bound = np.abs(A).max(1)[:, None] * np.abs(B).sum(1)[None, :] + \
        np.abs(A).sum(1)[:, None] * np.abs(B).max(1)[None, :]
    err = np.abs(C - ref)
    assert np.all(err <= 2e-15 * bound + 1e-300), float((err / bound).max())


def oz_s(A, B, slices):
    import torch
    from flare_gb300 import _lib
    M, K = A.shape
    N = B.shape[0]
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    dC = torch.full((max(M, 1), max(N, 1)), np.nan, dtype=torch.float64,
                    device="cuda")
    _lib.check(_lib.lib().fgb_oz_dgemm_nt_slices(
        slices, M, N, K, _lib.ptr(dA), K, _lib.ptr(dB), K, _lib.ptr(dC),
        max(N, 1), _lib.stream_ptr()))
    torch.cuda.synchronize()
    return dC.cpu().numpy()[:M, :N]


def emulate(A, B, S):
    """Exact emulation of the S-slice product: per-row power-of-two scales,
    X = rn(y 2^(6S)), balanced base-64 digits, the digit products with
    a + b <= S + 1 summed exactly (integers below 2^53 in FP64), one final
    rounding."""
    from fractions import Fraction

    def digits(X):
        e = np.frexp(np.abs(X).max(1))[1].astype(np.int64)
        Y = np.rint(np.ldexp(X, (6 * S - e)[:, None])).astype(np.int64)
        bias = sum(32 << (6 * (S - a)) for a in range(2, S + 1))
        U = Y + bias
        d = [(U >> (6 * (S - 1))).astype(np.float64)]
        for a in range(2, S + 1):
            d.append((((U >> (6 * (S - a))) & 63) - 32).astype(np.float64))
        return d, e

    da, ea = digits(A)
    db, eb = digits(B)
    G = []
    for t in range(2, S + 2):
        g = np.zeros((A.shape[0], B.shape[0]))
        for a in range(1, S + 1):
            if 1 <= t - a <= S:
                g += da[a - 1] @ db[t - a - 1].T
        G.append(g)
    out = np.zeros((A.shape[0], B.shape[0]))
    for i in range(A.shape[0]):
        for j in range(B.shape[0]):
            v = sum(Fraction(int(G[t - 2][i, j])) / (1 << (6 * t))
                    for t in range(2, S + 2))
            out[i, j] = float(v * Fraction(2) ** int(ea[i] + eb[j]))
    return out


@pytest.mark.parametrize("S", [8, 7])
def test_fewer_slices_match_exact_emulation(S):
    """8 and 7 slices (the mixed path's kernel and variance GEMMs): the
    result is the exactly rounded value of the truncated digit sum, so it
    equals an exact CPU emulation bit for bit."""
    r = np.random.Generator(np.random.PCG64(100 + S))
    A = r.normal(size=(40, 96)) * np.exp(r.uniform(-4, 1, size=(40, 96)))
    B = r.normal(size=(24, 96)) * np.exp(r.uniform(-4, 1, size=(24, 96)))
    np.testing.assert_array_equal(oz_s(A, B, S), emulate(A, B, S))


@pytest.mark.parametrize("S", [8, 7])
@pytest.mark.parametrize("M,N,K", [(300, 130, 680), (257, 1000, 1000)])
def test_fewer_slices_error_bound(S, M, N, K):
    """At S slices the dropped digit products and the slice residuals stay
    below 2^(-6S) (2^-48, 2^-42) of the row maxima: |C - A B^T| <=
    2 2^(-6S) (max|A_i| sum|B_j| + sum|A_i| max|B_j|)."""
    r = np.random.Generator(np.random.PCG64(M + N + S))
    A = r.normal(size=(M, K)) * np.exp(r.uniform(-6, 2, size=(M, K)))
    B = r.normal(size=(N, K)) * np.exp(r.uniform(-6, 2, size=(N, K)))
    C = oz_s(A, B, S)
    ref = A @ B.T
    bound = np.abs(A).max(1)[:, None] * np.abs(B).sum(1)[None, :] + \
        np.abs(A).sum(1)[:, None] * np.abs(B).max(1)[None, :]
    err = np.abs(C - ref)
    assert np.all(err <= 2.0 ** (1 - 6 * S) * bound + 2e-16 * np.abs(ref)), \
        float((err / bound).max())
    # and the error is not far below the bound: the slices are really cut
    assert (err / bound).max() > 2.0 ** (-6 * S - 12)


def test_slices_9_equals_default_entry():
    r = np.random.Generator(np.random.PCG64(9))
    A = r.normal(size=(130, 200))
    B = r.normal(size=(70, 200))
    np.testing.assert_array_equal(oz_s(A, B, 9), oz(A, B))


def oz32(A, B):
    import torch
    from flare_gb300 import _lib
    M, K = A.shape
    N = B.shape[0]
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    dC = torch.full((max(M, 1), max(N, 1)), np.nan, dtype=torch.float32,
                    device="cuda")
    _lib.check(_lib.lib().fgb_oz_sgemm_nt(M, N, K, _lib.ptr(dA), K,
                                          _lib.ptr(dB), K, _lib.ptr(dC),
                                          max(N, 1), _lib.stream_ptr()))
    torch.cuda.synchronize()
    return dC.cpu().numpy()[:M, :N].astype(np.float64)


@pytest.mark.parametrize("M,N,K", [(128, 128, 16), (300, 200, 680),
                                   (1000, 385, 385), (5, 3, 17)])
def test_fp32_level_accuracy(M, N, K):
    """4-slice configuration: the dropped digit products and slice residuals
    are below 2^-24 of the row maxima, and the result is rounded once to
    FP32."""
    r = np.random.Generator(np.random.PCG64(M + 3 * N))
    A = r.normal(size=(M, K)) * np.exp(r.uniform(-3, 1, size=(M, K)))
    B = r.normal(size=(N, K)) * np.exp(r.uniform(-3, 1, size=(N, K)))
    C = oz32(A, B)
    ref = A @ B.T
    bound = np.abs(A).max(1)[:, None] * np.abs(B).sum(1)[None, :] + \
        np.abs(A).sum(1)[:, None] * np.abs(B).max(1)[None, :]
    err = np.abs(C - ref)
    assert np.all(err <= 2.0 ** -22 * bound + 2.0 ** -24 * np.abs(ref)), \
        float((err / bound).max())


def test_fp32_level_integer_products_exact():
    """Integers of at most 24 bits in 4 digits: products exact, sums exact,
    and small enough to be exact in FP32."""
    r = np.random.Generator(np.random.PCG64(5))
    A = r.integers(-1000, 1001, size=(130, 256)).astype(np.float64)
    B = r.integers(-30, 31, size=(140, 256)).astype(np.float64)
    C = oz32(A, B)
    exact = (A.astype(np.int64) @ B.astype(np.int64).T).astype(np.float64)
    assert np.abs(exact).max() < 2 ** 24
    np.testing.assert_array_equal(C, exact)


def test_fp32_level_k_segments():
    """FP32-level configuration past its segment length (2720)."""
    r = np.random.Generator(np.random.PCG64(77))
    K = 6000
    A = r.normal(size=(140, K))
    B = r.normal(size=(130, K))
    C = oz32(A, B)
    ref = A @ B.T
    bound = np.abs(A).max(1)[:, None] * np.abs(B).sum(1)[None, :] + \
        np.abs(A).sum(1)[:, None] * np.abs(B).max(1)[None, :]
    err = np.abs(C - ref)
    assert np.all(err <= 2.0 ** -22 * bound + 2.0 ** -24 * np.abs(ref))
