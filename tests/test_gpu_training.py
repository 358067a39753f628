"""GPU: the reference-algorithm pieces — stored-gradient envs_struc,
envs_envs, Kuu/Kuf bookkeeping and the FP64 QR solve — against the oracle,
and the plain FP64 prediction form."""
import numpy as np
import pytest

import oracle
from helpers import b2_args, lj_labels, random_atoms, small_two_species

pytestmark = pytest.mark.gpu


def _train_both(seed=0, n_train=2, multicut=False, stress=True):
    import flare_gb300 as fg
    S = 2
    cutoffs = (5.0 * np.ones((S, S)) + np.eye(S) - 1) if multicut else None
    b2a = b2_args(S, 3, 2, 5.0, cutoffs=cutoffs)
    ob2 = oracle.B2Settings(*b2a)
    gb2 = fg.B2(*b2a[:5], cutoffs=cutoffs)
    ogp = oracle.SparseGP([oracle.NormalizedDotProduct(1.5, 2)], 0.3, 0.2, 0.4)
    ggp = fg.SparseGP([fg.NormalizedDotProduct(1.5, 2)], 0.3, 0.2, 0.4)
    r = np.random.Generator(np.random.PCG64(seed))
    for t in range(n_train):
        cell, sp, pos = random_atoms(seed=seed * 10 + t)
        E, F, St = lj_labels(cell, sp, pos, S)
        atoms = sorted(r.choice(len(sp), size=4, replace=False).tolist())
        o = oracle.Structure(cell, sp, pos, 5.0, [ob2])
        g = fg.Structure(cell, sp, pos, 5.0, [gb2])
        for s in (o, g):
            s.energy = np.array([E])
            s.forces = F.reshape(-1)
            if stress:
                s.stresses = St
        ogp.add_training_structure(o)
        ggp.add_training_structure(g)
        ogp.add_specific_environments(o, atoms)
        ggp.add_specific_environments(g, atoms)
    ogp.update_matrices_QR()
    ggp.update_matrices_QR()
    return ogp, ggp, b2a, gb2


@pytest.mark.parametrize("multicut", [False, True])
def test_envs_struc_matches_oracle(multicut):
    import flare_gb300 as fg
    ogp, b2a = small_two_species(seed=8, n_train=2, multicut=multicut)
    cutoffs = b2a[5]
    cell, sp, pos = random_atoms(seed=88)
    o = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    K0 = ogp.kernels[0].envs_struc(ogp.sparse_descriptors[0], o.descriptors[0])
    g = fg.Structure(cell, sp, pos, 5.0, [fg.B2(*b2a[:5], cutoffs=cutoffs)])
    sd = fg.ClusterDescriptor(2, ogp.sparse_descriptors[0].n_descriptors)
    osd = ogp.sparse_descriptors[0]
    sd.descriptors = [np.asarray(d) for d in osd.descriptors]
    sd.descriptor_norms = [np.asarray(d) for d in osd.descriptor_norms]
    sd.n_clusters_by_type = list(osd.n_clusters_by_type)
    sd.cumulative_type_count = list(osd.cumulative_type_count)
    sd.n_clusters = osd.n_clusters
    K1 = fg.NormalizedDotProduct(ogp.kernels[0].sigma, 2).envs_struc(sd, g)
    np.testing.assert_allclose(K1, K0, rtol=1e-9, atol=1e-9 * np.abs(K0).max())


@pytest.mark.parametrize("multicut", [False, True])
def test_training_matches_oracle(multicut):
    ogp, ggp, b2a, gb2 = _train_both(seed=3, multicut=multicut)
    np.testing.assert_allclose(ggp.Kuu, ogp.Kuu, rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(ggp.Kuf, ogp.Kuf, rtol=1e-9,
                               atol=1e-9 * np.abs(ogp.Kuf).max())
    np.testing.assert_allclose(ggp.y, ogp.y)
    np.testing.assert_allclose(ggp.noise_vector, ogp.noise_vector)
    np.testing.assert_allclose(ggp.L_inv, ogp.L_inv, rtol=1e-8,
                               atol=1e-8 * np.abs(ogp.L_inv).max())
    # alpha is ill-conditioned; compare predictions instead of raw alpha
    import flare_gb300 as fg
    cell, sp, pos = random_atoms(seed=99)
    o = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    ogp.predict_mean(o)
    g = fg.Structure(cell, sp, pos, 5.0, [gb2])
    ggp.predict_mean(g)
    scale = np.abs(o.mean_efs).max()
    np.testing.assert_allclose(g.mean_efs, o.mean_efs, atol=1e-6 * scale)


def test_plain_form_matches_fused_path():
    """The plain FP64 GPU form (stored gradients, envs_struc, K^T alpha)
    and the fused adjoint path give the same E/F/S and variances."""
    import ctypes
    import torch
    import flare_gb300 as fg
    from flare_gb300 import _lib
    from helpers import to_gpu_sgp
    ogp, b2a = small_two_species(seed=4, n_train=2)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    cell, sp, pos = random_atoms(seed=44)
    g = fg.Structure(cell, sp, pos, 5.0, [calc])
    fused = ggp.predict_batch([g])
    m = ggp._device_model([calc])
    N = g.noa
    mean = torch.zeros(1 + 3 * N + 6, dtype=torch.float64, device="cuda")
    var = torch.zeros(N, dtype=torch.float64, device="cuda")
    d = g._inputs()
    _lib.check(_lib.lib().fgb_predict_plain(m.h, g.nlist().h,
                                            _lib.ptr(d["species"]),
                                            _lib.ptr(mean), _lib.ptr(var),
                                            _lib.stream_ptr()))
    mean = mean.cpu().numpy()
    scale = max(1.0, abs(mean[0]))
    assert abs(mean[0] - fused["energy"][0]) < 1e-9 * scale
    np.testing.assert_allclose(mean[1:-6].reshape(-1, 3), fused["forces"],
                               atol=1e-8)
    np.testing.assert_allclose(mean[-6:], fused["stress"][0], atol=1e-10)
    np.testing.assert_allclose(var.cpu().numpy(), fused["local_var"],
                               atol=1e-12)


def test_batched_environment_addition_matches_sequential():
    """add_environments_batch gives the Kuu, Kuf, sparse set and weights of
    the same add_specific_environments calls made one by one."""
    import flare_gb300 as fg
    S = 2
    b2a = b2_args(S, 3, 2, 5.0)
    gb2 = fg.B2(*b2a[:5])
    gps = [fg.SparseGP([fg.NormalizedDotProduct(1.5, 2)], 0.3, 0.2, 0.4)
           for _ in range(2)]
    strucs = []
    for t in range(3):
        cell, sp, pos = random_atoms(seed=70 + t)
        E, F, St = lj_labels(cell, sp, pos, S)
        st = fg.Structure(cell, sp, pos, 5.0, [gb2])
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        st.stresses = St
        strucs.append(st)
    for gp in gps:
        for st in strucs[:2]:
            gp.add_training_structure(st)
            gp.add_specific_environments(st, [0, 3])
    picks = [(strucs[0], [1, 5]), (strucs[2], [2, 4, 6]), (strucs[1], [7])]
    for st, atoms in picks:
        gps[0].add_specific_environments(st, atoms)
    gps[1].add_environments_batch(picks)
    for gp in gps:
        gp.update_matrices_QR()
    a, b = gps
    assert a.n_sparse == b.n_sparse
    np.testing.assert_allclose(b.Kuu, a.Kuu, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(b.Kuf, a.Kuf, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(b.alpha, a.alpha, rtol=1e-9, atol=1e-9)
    for s in range(S):
        np.testing.assert_array_equal(b.sparse_descriptors[0].descriptors[s],
                                      a.sparse_descriptors[0].descriptors[s])


def test_set_hyperparameters_matches_fresh_model():
    """ctests/test_sparse_gp.cpp:300-366 (Set_Hyps): two GPs on the same
    data with different hyperparameters and per-structure relative noises;
    after set_hyperparameters(hyps of the first) the second has the first's
    Kuu, Kuf, noise vector, alpha and predictions."""
    import flare_gb300 as fg
    b2a = b2_args(2, 3, 2, 5.0)
    gb2 = fg.B2(*b2a[:5])
    gps = [fg.SparseGP([fg.NormalizedDotProduct(1.5, 2)], 1.0, 1.5, 3.0),
           fg.SparseGP([fg.NormalizedDotProduct(2.0, 2)], 2.0, 2.5, 3.5)]
    rel = [(0.1, 0.2, 0.3), (0.5, 0.4, 0.6)]
    for t in range(2):
        cell, sp, pos = random_atoms(seed=70 + t)
        E, F, St = lj_labels(cell, sp, pos, 2)
        for gp in gps:
            g = fg.Structure(cell, sp, pos, 5.0, [gb2])
            g.energy, g.forces, g.stresses = np.array([E]), F.reshape(-1), St
            gp.add_training_structure(g, [-1], *rel[t])
            gp.add_all_environments(g)
    for gp in gps:
        gp.update_matrices_QR()
    assert not np.allclose(gps[0].alpha, gps[1].alpha)
    gps[1].set_hyperparameters(gps[0].hyperparameters)
    np.testing.assert_allclose(gps[1].hyperparameters, gps[0].hyperparameters)
    np.testing.assert_allclose(gps[1].Kuu, gps[0].Kuu, rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(gps[1].Kuf, gps[0].Kuf, rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(gps[1].noise_vector, gps[0].noise_vector,
                               rtol=1e-14)
    np.testing.assert_allclose(gps[1].alpha, gps[0].alpha, rtol=1e-7,
                               atol=1e-7 * np.abs(gps[0].alpha).max())
    cell, sp, pos = random_atoms(seed=79)
    r = [gp.predict_batch([fg.Structure(cell, sp, pos, 5.0, [gb2])])
         for gp in gps]
    np.testing.assert_allclose(r[1]["forces"], r[0]["forces"], rtol=0,
                               atol=1e-7 * max(1, np.abs(r[0]["forces"]).max()))
