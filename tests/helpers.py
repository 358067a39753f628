"""Shared test fixtures: oracle-trained models and converters.

Models are trained by the FP64 oracle (oracle/oracle.py) and installed into
the GPU SparseGP, so GPU prediction is compared with the oracle on the same
weights.
"""
import numpy as np

import oracle
from flare_gb300 import synthetic as syn


def rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def random_atoms(a=2.0, sc=2, numbers=(0, 1), seed=0):
    """2-atom basis, sc^3 supercell, jitter +-0.1 (the reference fixture
    tests/get_sgp.py:23-38 with a seeded generator)."""
    r = rng(seed)
    basis = np.array([[0, 0, 0], r.uniform(size=3) * a])
    g = np.stack(np.meshgrid(*[np.arange(sc)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pos = (g[:, None, :] * a + basis[None]).reshape(-1, 3)
    species = np.tile(np.asarray(numbers), len(g))
    pos = pos + (2 * r.uniform(size=pos.shape) - 1) * 0.1
    return np.eye(3) * a * sc, species, pos


def b2_args(S=1, nmax=8, lmax=3, rc=5.0, cutoff_function="quadratic",
            cutoffs=None):
    return ("chebyshev", cutoff_function, [0.0, rc], [], [S, nmax, lmax],
            cutoffs)


def oracle_model(strucs, labels, sparse, b2a, sigma=2.0, power=2,
                 noise=(0.1, 0.05, 0.1), cutoff=5.0):
    """Train an oracle SparseGP: strucs = [(cell, species, pos)], labels =
    [(E, F, S or None)], sparse = [list of atom indices per structure]."""
    b2 = oracle.B2Settings(*b2a)
    k = oracle.NormalizedDotProduct(sigma, power)
    gp = oracle.SparseGP([k], *noise)
    for (cell, sp, pos), (E, F, St), atoms in zip(strucs, labels, sparse):
        st = oracle.Structure(cell, sp, pos, cutoff, [b2])
        st.energy = np.array([E])
        st.forces = np.asarray(F).reshape(-1)
        if St is not None:
            st.stresses = np.asarray(St)
        gp.add_training_structure(st)
        gp.add_specific_environments(st, atoms)
    gp.update_matrices_QR()
    return gp, b2


def to_gpu_sgp(ogp, b2a, cutoff=5.0):
    """GPU SparseGP carrying the oracle model's weights."""
    import flare_gb300 as fg
    calc = fg.B2(*b2a[:5], cutoffs=b2a[5])
    k = fg.NormalizedDotProduct(ogp.kernels[0].sigma, ogp.kernels[0].power)
    gp = fg.SparseGP([k], ogp.energy_noise, ogp.force_noise, ogp.stress_noise)
    osd = ogp.sparse_descriptors[0]
    cd = fg.ClusterDescriptor(osd.n_types, osd.n_descriptors)
    cd.descriptors = [np.asarray(d) for d in osd.descriptors]
    cd.descriptor_norms = [np.asarray(d) for d in osd.descriptor_norms]
    cd.n_clusters_by_type = list(osd.n_clusters_by_type)
    cd.cumulative_type_count = list(osd.cumulative_type_count)
    cd.n_clusters = osd.n_clusters
    gp.set_weights([cd], ogp.alpha, ogp.L_inv, [calc])
    return gp, calc


def lj_labels(cell, sp, pos, S=1):
    eps = [0.4, 0.25, 0.3][:S]
    sig = [2.6, 2.3, 2.45][:S]
    return syn.lennard_jones(cell, sp, pos, eps, sig, 5.0)


def small_two_species(seed=0, n_train=3, power=2, multicut=False):
    """Reference-fixture-like model: 2 species, B2 [2, 3, 2], rc 5.0, a=2.0
    2x2x2 cells (tiny box: several image shells)."""
    S = 2
    cutoffs = None
    if multicut:
        cutoffs = 5.0 * np.ones((S, S)) + np.eye(S) - 1
    b2a = b2_args(S, 3, 2, 5.0, cutoffs=cutoffs)
    r = rng(seed)
    strucs, labels, sparse = [], [], []
    for t in range(n_train):
        cell, sp, pos = random_atoms(seed=seed * 100 + t)
        strucs.append((cell, sp, pos))
        labels.append(lj_labels(cell, sp, pos, S))
        sparse.append(sorted(r.choice(len(sp), size=5, replace=False).tolist()))
    gp, b2 = oracle_model(strucs, labels, sparse, b2a, sigma=1.5, power=power,
                          noise=(0.3, 0.2, 0.4))
    return gp, b2a


def c1_model(n_train=20, n_sparse=200, power=2):
    """FCC Al-like model of the 256-atom workload (seeded)."""
    b2a = b2_args(1, 8, 3, 5.0)
    strucs, labels = [], []
    for s in range(1000, 1000 + n_train):
        cell, sp, pos = syn.fcc_al(seed=s)
        strucs.append((cell, sp, pos))
        E, F, _ = lj_labels(cell, sp, pos, 1)
        labels.append((E, F, None))
    chosen = rng(1200).choice(n_train * 256, size=n_sparse, replace=False)
    sparse = [sorted(int(c) - 256 * i for c in chosen if c // 256 == i)
              for i in range(n_train)]
    gp, b2 = oracle_model(strucs, labels, sparse, b2a, sigma=2.0, power=power,
                          noise=(0.256, 0.05, 1.0))
    return gp, b2a


def alloy_oracle_model(n_train=2):
    """Oracle SparseGP of the alloy1000 workload (flare_gb300.workloads):
    2 species, B2 [2, 8, 4], rc 5.5 A, NormalizedDotProduct sigma 2 power
    2, trained on the first ``n_train`` training structures with LJ energy
    and force labels and the workload's sparse choice (about 1,000 sparse
    environments per species)."""
    from flare_gb300 import workloads as wl
    c = wl.ALLOY
    b2a = b2_args(2, c["n_max"], c["l_max"], c["rc"])
    data = [wl.alloy_structure(c["train_seed0"] + t) for t in range(n_train)]
    sparse = wl.alloy_sparse_choice(n_train, [d[1] for d in data],
                                    c["sparse_per_species"], c["sparse_seed"])
    labels = []
    for cell, sp, pos in data:
        E, F, _ = wl.alloy_labels(cell, sp, pos)
        labels.append((E, F, None))
    gp, _ = oracle_model(data, labels, sparse, b2a, sigma=c["sigma"],
                         power=c["power"],
                         noise=(c["sigma_e_per_atom"] * c["n_atoms"],
                                c["sigma_f"], c["sigma_s"]),
                         cutoff=c["rc"])
    return gp, b2a
