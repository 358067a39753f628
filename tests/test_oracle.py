"""CPU: the oracle against the reference's golden vectors and the
relations the reference's own tests check."""
import os

import numpy as np
import pytest

import oracle
from helpers import b2_args, random_atoms, small_two_species
from flare_gb300 import synthetic as syn

GOLD = os.path.join(os.path.dirname(__file__), "golden", "per_pair.npz")


def test_ylm_matches_reference_golden():
    """y_grad.cpp get_Y values and gradients, l <= 10 (golden from the
    reference's compiled source)."""
    g = np.load(GOLD)
    L = int(g["ylm_lmax"])
    for i, p in enumerate(g["ylm_points"]):
        mine = np.stack(oracle.ylm(*p, L))
        ref = g["ylm"][i]
        np.testing.assert_allclose(mine, ref, rtol=1e-12,
                                   atol=1e-13 * max(1, np.abs(ref).max()))


@pytest.mark.parametrize("cut", ["quadratic", "hard", "cosine", "polynomial",
                                 "power"])
def test_radial_matches_reference_golden(cut):
    """calculate_radial (radial.cpp:344) with the Chebyshev basis."""
    g = np.load(GOLD)
    for i, p in enumerate(g["radial_points"]):
        mine = np.stack(oracle.radial(
            "chebyshev", cut, *p, g["radial_r"][i], float(g["radial_rcut"]),
            int(g["radial_nmax"]), 0.0, list(g["cutoff_hyps_" + cut])))
        np.testing.assert_array_equal(mine, g["radial_" + cut][i])


BASES = ["chebyshev", "weighted_chebyshev", "equispaced_gaussians",
         "weighted_positive_chebyshev", "positive_chebyshev", "bessel",
         "fourier_quarter", "fourier_half", "fourier"]


@pytest.mark.parametrize("basis", BASES)
def test_radial_bases_match_reference_golden(basis):
    """Every radial basis (radial.cpp:6-336) times the quadratic cutoff,
    against the reference's own compiled functions; the same operations in
    the same order, so within a few units of the last place."""
    g = np.load(GOLD)
    rh = list(g["basis_hyps_" + basis])
    ref = g["basis_" + basis]
    for i, p in enumerate(g["radial_points"]):
        mine = np.stack(oracle.radial(
            basis, "quadratic", *p, g["radial_r"][i], rh[1],
            int(g["radial_nmax"]), rh[0], [], rh[2] if len(rh) > 2 else 0.0))
        np.testing.assert_allclose(mine, ref[i], rtol=1e-13,
                                   atol=1e-13 * max(1.0, np.abs(ref[i]).max()))


def test_ylm_gradient_finite_difference():
    """test_y_grad.cpp: gradients against central differences."""
    r = np.random.Generator(np.random.PCG64(5))
    for _ in range(10):
        p = r.normal(size=3)
        Y, Yx, Yy, Yz = oracle.ylm(*p, 6)
        h = 1e-6
        for k, G in enumerate([Yx, Yy, Yz]):
            dp = np.zeros(3)
            dp[k] = h
            fd = (oracle.ylm(*(p + dp), 6)[0] - oracle.ylm(*(p - dp), 6)[0]) / (2 * h)
            np.testing.assert_allclose(G, fd, atol=1e-7)


def _rot(seed):
    q, _ = np.linalg.qr(np.random.Generator(np.random.PCG64(seed)).normal(size=(3, 3)))
    return q


def test_b2_rotation_invariance():
    """test_descriptor.cpp:49-69: B2 invariant under rotation (1e-10)."""
    cell, sp, pos = random_atoms(seed=3)
    b2 = oracle.B2Settings(*b2_args(2, 4, 3, 5.0))
    R = _rot(1)
    s1 = oracle.Structure(cell, sp, pos, 5.0, [b2], compute_dervs=False)
    s2 = oracle.Structure(cell @ R, sp, pos @ R, 5.0, [b2], compute_dervs=False)
    np.testing.assert_allclose(s1.descriptors[0].atom_B2,
                               s2.descriptors[0].atom_B2, rtol=1e-10, atol=1e-10)


def test_neighbor_list_symmetric():
    cell, sp, pos = syn.fcc_al(n_cells=2, seed=4)
    s = oracle.Structure(cell, sp, pos, 5.0, [])
    pairs = set()
    off = s.cumulative_neighbor_count
    for i in range(s.noa):
        for p in range(off[i], off[i + 1]):
            pairs.add((i, int(s.structure_indices[p]), tuple(s.shifts[p])))
    for (i, j, sh) in pairs:
        assert (j, i, tuple(-np.asarray(sh))) in pairs


def test_envs_sum_equals_energy_kernel():
    """test_kernels.cpp:35-75 relation: the energy column of envs_struc is
    the sum of envs_envs over the structure's atoms."""
    gp, b2a = small_two_species(seed=1, n_train=1)
    k = gp.kernels[0]
    cell, sp, pos = random_atoms(seed=77)
    st = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    K = k.envs_struc(gp.sparse_descriptors[0], st.descriptors[0])
    cd = oracle.ClusterDescriptor.from_values(st.descriptors[0])
    Kee = k.envs_envs(gp.sparse_descriptors[0], cd)
    np.testing.assert_allclose(K[:, 0], Kee.sum(1), rtol=1e-10, atol=1e-10)


def test_force_and_stress_columns_finite_difference():
    """test_kernels.cpp:140-400: force/stress kernel columns against central
    differences of the energy column (delta 1e-4, tolerance 1e-4)."""
    gp, b2a = small_two_species(seed=2, n_train=1)
    k = gp.kernels[0]
    b2 = oracle.B2Settings(*b2a)
    cell, sp, pos = random_atoms(seed=9)
    st = oracle.Structure(cell, sp, pos, 5.0, [b2])
    K = k.envs_struc(gp.sparse_descriptors[0], st.descriptors[0])
    d = 1e-4
    for atom in [0, 5]:
        for c in range(3):
            p1 = pos.copy(); p1[atom, c] += d
            p2 = pos.copy(); p2[atom, c] -= d
            e1 = k.envs_struc(gp.sparse_descriptors[0], oracle.Structure(
                cell, sp, p1, 5.0, [b2]).descriptors[0])[:, 0]
            e2 = k.envs_struc(gp.sparse_descriptors[0], oracle.Structure(
                cell, sp, p2, 5.0, [b2]).descriptors[0])[:, 0]
            np.testing.assert_allclose(K[:, 1 + 3 * atom + c],
                                       -(e1 - e2) / (2 * d), atol=1e-4)
    # stress xx: strain the cell and positions together
    eps = np.eye(3)
    eps[0, 0] += d
    e1 = k.envs_struc(gp.sparse_descriptors[0], oracle.Structure(
        cell @ eps, sp, pos @ eps, 5.0, [b2]).descriptors[0])[:, 0]
    eps[0, 0] -= 2 * d
    e2 = k.envs_struc(gp.sparse_descriptors[0], oracle.Structure(
        cell @ eps, sp, pos @ eps, 5.0, [b2]).descriptors[0])[:, 0]
    vol = abs(np.linalg.det(cell))
    np.testing.assert_allclose(K[:, 1 + 3 * st.noa], -(e1 - e2) / (2 * d) / vol,
                               atol=1e-4)


def test_local_variances_nonnegative_and_sparse_points_small():
    """test_sparse_gp.cpp:55-119: variances >= 0 (to rounding)."""
    gp, b2a = small_two_species(seed=3, n_train=2)
    cell, sp, pos = random_atoms(seed=123)
    st = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    v = gp.compute_cluster_uncertainties(st)[0]
    assert np.all(v > -1e-8)


def test_model_from_weights_predicts_the_same():
    """SparseGP.from_weights (the oracle carrying another model's weights)
    predicts exactly what the trained model predicts."""
    gp, b2a = small_two_species(seed=4, n_train=2)
    twin = oracle.SparseGP.from_weights(gp.kernels, gp.sparse_descriptors,
                                        gp.alpha, gp.L_inv)
    cell, sp, pos = random_atoms(seed=77)
    a = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    b = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    gp.predict_local_uncertainties(a)
    twin.predict_local_uncertainties(b)
    np.testing.assert_array_equal(a.mean_efs, b.mean_efs)
    np.testing.assert_array_equal(a.local_uncertainties[0],
                                  b.local_uncertainties[0])


def _unit_rows(st):
    dv = st.descriptors[0]
    out = []
    for s in range(dv.n_types):
        D, n = dv.descriptors[s], dv.descriptor_norms[s]
        ok = n >= 1e-8
        U = np.zeros_like(D)
        U[ok] = D[ok] / n[ok, None]
        out.append(U)
    return out


@pytest.mark.parametrize("power", [1, 2])
def test_self_kernel_struc_finite_difference(power):
    """self_kernel_struc (normalized_dot_product.cpp:450-586) is the diagonal
    of the structure-structure kernel: the energy entry equals
    sigma^2 sum_ij c_ij^power, a force entry the mixed second derivative of
    that sum with respect to one atom's coordinate in each structure, a
    stress entry the mixed second derivative with respect to the
    deformation x_m += h x_n of each cell, over V^2.  Four-point central
    differences, h = 3e-4 (truncation ~1e-6 relative, rounding ~1e-7
    absolute)."""
    b2a = b2_args(2, 3, 2, 4.0)
    b2 = oracle.B2Settings(*b2a)
    cell, sp, pos = random_atoms(seed=7)
    sig = 1.5
    k = oracle.NormalizedDotProduct(sig, power)
    st = oracle.Structure(cell, sp, pos, 4.0, [b2])
    K = k.self_kernel_struc(st.descriptors[0])
    n = len(sp)
    assert K.shape == (1 + 3 * n + 6,)

    def rows(c, p):
        return _unit_rows(oracle.Structure(c, sp, p, 4.0, [b2],
                                           compute_dervs=False))

    def kee(A, B):
        return sig * sig * sum(float(np.sum((a @ b.T) ** power))
                               for a, b in zip(A, B))

    U0 = rows(cell, pos)
    assert abs(K[0] - kee(U0, U0)) <= 1e-12 * abs(K[0])
    h = 3e-4
    for a, m in [(0, 0), (3, 1), (9, 2), (14, 0)]:
        P = []
        for d in (h, -h):
            q = pos.copy()
            q[a, m] += d
            P.append(rows(cell, q))
        fd = (kee(P[0], P[0]) - kee(P[0], P[1]) - kee(P[1], P[0]) +
              kee(P[1], P[1])) / (4 * h * h)
        assert abs(K[1 + 3 * a + m] - fd) <= 2e-5 * abs(fd) + 1e-6, (a, m)
    vol = abs(np.linalg.det(cell))
    for c, (m, nn) in enumerate([(0, 0), (0, 1), (0, 2), (1, 1), (1, 2),
                                 (2, 2)]):
        # a stretch moves pairs across the cutoff, whose quadratic form has
        # a jump in the second derivative: the difference then converges
        # only linearly in h, so diagonal entries use a smaller step
        hs = 1e-5 if m == nn else h
        P = []
        for d in (hs, -hs):
            F = np.eye(3)
            F[m, nn] += d
            P.append(rows(cell @ F.T, pos @ F.T))
        fd = (kee(P[0], P[0]) - kee(P[0], P[1]) - kee(P[1], P[0]) +
              kee(P[1], P[1])) / (4 * hs * hs) / vol ** 2
        assert abs(K[1 + 3 * n + c] - fd) <= 2e-5 * abs(fd) + 1e-8, (m, nn)


def test_predict_dtc_variances_relation():
    """predict_DTC (sparse_gp.cpp:694-729) against its definition assembled
    from the oracle's own parts, and SOR's variances plus K_self -
    diag(K^T Kuu^-1 K)."""
    ogp, b2a = small_two_species(seed=5, n_train=2)
    cell, sp, pos = random_atoms(seed=55)
    st = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    ogp.predict_DTC(st)
    dtc = st.variance_efs.copy()
    ogp.predict_SOR(st)
    sor = st.variance_efs.copy()
    km = ogp._kernel_mat(st)
    ks = ogp.kernels[0].self_kernel_struc(st.descriptors[0])
    q = np.einsum("ij,ij->j", km, ogp.Kuu_inverse @ km)
    np.testing.assert_allclose(dtc, ks - q + sor,
                               atol=1e-9 * np.abs(ks).max())


def test_struc_struc_relations():
    """struc_struc (normalized_dot_product.cpp:216-448) against the
    reference's own kernel tests (ctests/test_kernels.cpp): the energy entry
    is the sum of envs_envs over all atom pairs (:35-53), row 0 the column
    sums of envs_struc (:55-75), the matrix of (s2, s1) the transpose of
    (s1, s2), and force and stress entries the first and mixed second
    differences of the energy entry under atom moves and cell strains
    (:140-760; delta 1e-4 for first and 3e-4 for mixed second
    differences)."""
    b2 = oracle.B2Settings(*b2_args(2, 3, 2, 4.0))
    k = oracle.NormalizedDotProduct(1.5, 2)
    (c1, sp1, p1), (c2, sp2, p2) = random_atoms(seed=3), random_atoms(seed=4)
    sp2 = sp2[::-1].copy()
    st = lambda c, s, p, d=True: oracle.Structure(c, s, p, 4.0, [b2],
                                                   compute_dervs=d)
    s1, s2 = st(c1, sp1, p1), st(c2, sp2, p2)
    K = k.struc_struc(s1.descriptors[0], s2.descriptors[0])
    n1, n2 = len(sp1), len(sp2)
    assert K.shape == (1 + 3 * n1 + 6, 1 + 3 * n2 + 6)
    e1 = oracle.ClusterDescriptor.from_values(s1.descriptors[0])
    e2 = oracle.ClusterDescriptor.from_values(s2.descriptors[0])
    assert abs(K[0, 0] - k.envs_envs(e1, e2).sum()) < 1e-10 * abs(K[0, 0])
    np.testing.assert_allclose(k.envs_struc(e1, s2.descriptors[0]).sum(0),
                               K[0], rtol=0, atol=1e-10 * np.abs(K[0]).max())
    Kt = k.struc_struc(s2.descriptors[0], s1.descriptors[0])
    np.testing.assert_allclose(Kt.T, K, rtol=0, atol=1e-10 * np.abs(K).max())

    def ee(ca, pa, cb, pb):
        return k.struc_struc(st(ca, sp1, pa).descriptors[0],
                             st(cb, sp2, pb).descriptors[0])[0, 0]

    def move(p, a, m, d):
        q = p.copy()
        q[a, m] += d
        return q

    def strain(c, p, m, n, d):
        F = np.eye(3)
        F[m, n] += d
        return c @ F.T, p @ F.T

    h = 1e-4
    # energy / force (structure 2's atom 5, y) and force / energy
    fd = -(ee(c1, p1, c2, move(p2, 5, 1, h)) -
           ee(c1, p1, c2, move(p2, 5, 1, -h))) / (2 * h)
    assert abs(K[0, 1 + 3 * 5 + 1] - fd) < 1e-5 * max(1, abs(fd))
    fd = -(ee(c1, move(p1, 2, 0, h), c2, p2) -
           ee(c1, move(p1, 2, 0, -h), c2, p2)) / (2 * h)
    assert abs(K[1 + 3 * 2, 0] - fd) < 1e-5 * max(1, abs(fd))
    # energy / stress xy
    vol2 = abs(np.linalg.det(c2))
    fd = -(ee(c1, p1, *strain(c2, p2, 0, 1, h)) -
           ee(c1, p1, *strain(c2, p2, 0, 1, -h))) / (2 * h)
    assert abs(K[0, 1 + 3 * n2 + 1] * vol2 - fd) < 1e-5 * max(1, abs(fd))
    # mixed second differences: h = 3e-4 (rounding grows as 1/h^2)
    h = 3e-4
    # force / force
    for (a, m, b, n) in [(1, 0, 4, 2), (7, 2, 7, 2), (12, 1, 0, 0)]:
        P1 = [move(p1, a, m, d) for d in (h, -h)]
        P2 = [move(p2, b, n, d) for d in (h, -h)]
        fd = (ee(c1, P1[0], c2, P2[0]) + ee(c1, P1[1], c2, P2[1]) -
              ee(c1, P1[0], c2, P2[1]) - ee(c1, P1[1], c2, P2[0])) / (4 * h * h)
        got = K[1 + 3 * a + m, 1 + 3 * b + n]
        assert abs(got - fd) < 2e-5 * abs(fd) + 1e-6, (a, m, b, n, got, fd)
    # force / stress (atom 3 z of 1, yz of 2) and stress / stress (xz, xz)
    S2 = [strain(c2, p2, 1, 2, d) for d in (h, -h)]
    P1 = [move(p1, 3, 2, d) for d in (h, -h)]
    fd = (ee(c1, P1[0], *S2[0]) + ee(c1, P1[1], *S2[1]) -
          ee(c1, P1[0], *S2[1]) - ee(c1, P1[1], *S2[0])) / (4 * h * h)
    got = K[1 + 3 * 3 + 2, 1 + 3 * n2 + 4] * vol2
    assert abs(got - fd) < 2e-5 * abs(fd) + 1e-6, (got, fd)
    vol1 = abs(np.linalg.det(c1))
    S1 = [strain(c1, p1, 0, 2, d) for d in (h, -h)]
    S2 = [strain(c2, p2, 0, 2, d) for d in (h, -h)]
    fd = (ee(*S1[0], *S2[0]) + ee(*S1[1], *S2[1]) -
          ee(*S1[0], *S2[1]) - ee(*S1[1], *S2[0])) / (4 * h * h)
    got = K[1 + 3 * n1 + 2, 1 + 3 * n2 + 2] * vol1 * vol2
    assert abs(got - fd) < 2e-5 * abs(fd) + 1e-6, (got, fd)
