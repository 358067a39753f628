"""GPU: the FP64 dense kernels of the solve (update_matrices_QR,
sparse_gp.cpp:607-641) — blocked Cholesky, lower-triangular inverse and the
symmetric products Kuu^-1 = L_inv^T L_inv, Sigma = R_inv R_inv^T — against
numpy/LAPACK in FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spd(M, seed, cond=1e6):
    r = np.random.Generator(np.random.PCG64(seed))
    Q, _ = np.linalg.qr(r.normal(size=(M, M)))
    ev = np.geomspace(1.0, 1.0 / cond, M)
    return (Q * ev) @ Q.T


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def _chol(A):
    import torch
    from flare_gb300 import _lib
    d = _dev(A)
    _lib.check(_lib.lib().fgb_cholesky(A.shape[0], _lib.ptr(d),
                                       _lib.stream_ptr()), "cholesky")
    torch.cuda.synchronize()
    return d.cpu().numpy()


def _trtri(L):
    import torch
    from flare_gb300 import _lib
    d = _dev(L)
    x = torch.full_like(d, np.nan)
    _lib.check(_lib.lib().fgb_trtri_lower(L.shape[0], _lib.ptr(d), _lib.ptr(x),
                                          _lib.stream_ptr()), "trtri")
    torch.cuda.synchronize()
    return x.cpu().numpy()


@pytest.mark.parametrize("M", [1, 5, 128, 300, 1000, 3000])
def test_cholesky_matches_lapack(M):
    A = _spd(M, M)
    L = _chol(A)
    ref = np.linalg.cholesky(A)
    assert np.all(np.triu(L, 1) == 0.0)
    # backward error of the factorisation and the factor itself
    assert np.abs(L @ L.T - A).max() <= 1e-13 * np.abs(A).max() * np.sqrt(M)
    np.testing.assert_allclose(L, ref, rtol=0, atol=1e-9 * np.abs(ref).max())


def test_cholesky_reports_indefinite():
    A = _spd(200, 9)
    A[150, 150] = -1.0
    with pytest.raises(ValueError, match="not positive definite"):
        _chol(A)


@pytest.mark.parametrize("M", [1, 7, 128, 129, 640, 2000])
def test_trtri_matches_lapack(M):
    L = np.linalg.cholesky(_spd(M, 100 + M, cond=1e4))
    X = _trtri(L)
    assert np.all(np.triu(X, 1) == 0.0)
    ref = np.linalg.inv(L)
    # relative to the size of the inverse and its condition
    np.testing.assert_allclose(X @ L, np.eye(M), rtol=0,
                               atol=1e-12 * np.sqrt(M) * 1e2)
    np.testing.assert_allclose(X, ref, rtol=0, atol=1e-10 * np.abs(ref).max())


def test_solve_products():
    import torch
    from flare_gb300 import _lib
    M = 700
    r = np.random.Generator(np.random.PCG64(5))
    Li = np.tril(r.normal(size=(M, M)))
    Ri = np.triu(r.normal(size=(M, M)))
    dL, dR = _dev(Li), _dev(Ri)
    K = torch.empty_like(dL)
    S = torch.empty_like(dL)
    _lib.check(_lib.lib().fgb_solve_products(M, _lib.ptr(dL), _lib.ptr(dR),
                                             _lib.ptr(K), _lib.ptr(S),
                                             _lib.stream_ptr()), "products")
    torch.cuda.synchronize()
    def bound(A):   # C = A A^T: the exact-slicing GEMM's error bound
        mx, sm = np.abs(A).max(1), np.abs(A).sum(1)
        return np.outer(mx, sm) + np.outer(sm, mx)

    Kr, Sr = Li.T @ Li, Ri @ Ri.T
    assert np.all(np.abs(K.cpu().numpy() - Kr) <=
                  2e-15 * bound(Li.T) + 2e-16 * np.abs(Kr))
    assert np.all(np.abs(S.cpu().numpy() - Sr) <=
                  2e-15 * bound(Ri) + 2e-16 * np.abs(Sr))


def test_training_products_match_oracle():
    """Kuu_inverse and Sigma of a trained model (read from the GPU-formed
    products) against the oracle's numpy products."""
    from test_gpu_training import _train_both
    ogp, ggp, b2a, gb2 = _train_both(seed=6)
    np.testing.assert_allclose(ggp.Kuu_inverse, ogp.Kuu_inverse, rtol=0,
                               atol=1e-7 * np.abs(ogp.Kuu_inverse).max())
    np.testing.assert_allclose(ggp.Sigma, ogp.Sigma, rtol=0,
                               atol=1e-7 * np.abs(ogp.Sigma).max())
