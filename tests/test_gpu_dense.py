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


@pytest.mark.parametrize("M,nl,cond,rank,scale", [(300, 2000, 1e6, 300, 1.0),
                                                  (700, 5000, 1e10, 350, 1e-3)])
def test_solve_qr_matches_householder(M, nl, cond, rank, scale):
    """fgb_solve_qr (Cholesky, triangular inverses, shifted Cholesky QR)
    against numpy's Householder QR of the same A = [sqrt(noise) Kuf^T;
    L^T]: alpha, L_inv and Sigma = R_inv R_inv^T (R agrees up to row
    signs, so R_inv is compared through Sigma).  Kuf of rank `rank` scaled
    by `scale` leaves the small singular values to L^T: cond(A) = 1.9e4
    and 5.5e4."""
    import scipy.linalg as sla
    import torch
    from flare_gb300 import _lib
    r = np.random.Generator(np.random.PCG64(M + nl))
    Kuu = 4.0 * _spd(M, M + 1, cond=cond)
    Kuf = (r.normal(size=(M, rank)) @ r.normal(size=(rank, nl))) * scale / \
        np.sqrt(rank)
    y = r.normal(size=nl)
    noise = np.where(r.uniform(size=nl) < 0.1, 1e6, 400.0)
    jitter = 1e-8
    d = {k: _dev(v) for k, v in (("Kuu", Kuu), ("Kuf", Kuf), ("y", y),
                                   ("noise", noise))}
    alpha = torch.zeros(M, dtype=torch.float64, device="cuda")
    Li = torch.zeros((M, M), dtype=torch.float64, device="cuda")
    Ri = torch.zeros((M, M), dtype=torch.float64, device="cuda")
    _lib.check(_lib.lib().fgb_solve_qr(
        M, nl, _lib.ptr(d["Kuu"]), _lib.ptr(d["Kuf"]), _lib.ptr(d["y"]),
        _lib.ptr(d["noise"]), jitter, _lib.ptr(alpha), _lib.ptr(Li),
        _lib.ptr(Ri), _lib.stream_ptr()), "solve")
    torch.cuda.synchronize()
    Lc = np.linalg.cholesky(Kuu + jitter * np.eye(M))
    Lref = sla.solve_triangular(Lc, np.eye(M), lower=True)
    A = np.vstack([np.sqrt(noise)[:, None] * Kuf.T, Lc.T])
    b = np.concatenate([np.sqrt(noise) * y, np.zeros(M)])
    Q, R = np.linalg.qr(A)
    Rinv = sla.solve_triangular(R, np.eye(M), lower=False)
    aref = Rinv @ (Q.T @ b)
    Sref = Rinv @ Rinv.T
    Ri_ = Ri.cpu().numpy()
    # two backward-stable computations differ by up to about the problem's
    # condition number x u: cond(Kuu + jitter) for L_inv, cond(A)^2 for
    # alpha and Sigma = (A^T A)^-1
    ev = np.linalg.eigvalsh(Kuu + jitter * np.eye(M))
    tol_L = max(1e-9, 4 * (ev[-1] / ev[0]) * 2.0 ** -53)
    tol_a = max(1e-8, 10 * np.linalg.cond(A) ** 2 * 2.0 ** -53)
    np.testing.assert_allclose(Li.cpu().numpy(), Lref, rtol=0,
                               atol=tol_L * np.abs(Lref).max())
    np.testing.assert_allclose(alpha.cpu().numpy(), aref, rtol=0,
                               atol=tol_a * np.abs(aref).max())
    np.testing.assert_allclose(Ri_ @ Ri_.T, Sref, rtol=0,
                               atol=tol_a * np.abs(Sref).max())
    assert np.all(np.tril(Ri_, -1) == 0.0)
