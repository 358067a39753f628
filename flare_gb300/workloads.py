"""Named synthetic workloads with seeded inputs and GPU-trained models.

``alloy1000``: 2-species random alloy, 1,000-atom cubic cell at 0.06
atoms/A^3, species 50/50, 1.8 A minimum distance; B2 chebyshev/quadratic
n_max = 8, l_max = 4, rc = 5.5 A; NormalizedDotProduct sigma = 2, power = 2;
10 training structures (seeds 2000-2009) with truncated Lennard-Jones energy
and force labels (eps 0.4/0.25 eV, sigma 2.6/2.3 A, Lorentz-Berthelot
mixing); 1,000 sparse environments per species drawn without replacement
from the training pool (seed 2200); noise sigma_E = 1e-3 eV/atom (1.0 eV per
structure), sigma_F = 0.05 eV/A; test structures from seeds 2100, 2101, ...
"""
import numpy as np

from . import synthetic as syn

ALLOY = dict(n_atoms=1000, density=0.06, fractions=(0.5, 0.5), dmin=1.8,
             rc=5.5, n_max=8, l_max=4, sigma=2.0, power=2, eps=(0.4, 0.25),
             lj_sigma=(2.6, 2.3), n_train=10, train_seed0=2000,
             sparse_per_species=1000, sparse_seed=2200, test_seed0=2100,
             sigma_e_per_atom=1e-3, sigma_f=0.05, sigma_s=1.0)


def alloy_structure(seed, n_atoms=None):
    c = ALLOY
    return syn.random_alloy(n_atoms or c["n_atoms"], density=c["density"],
                            fractions=c["fractions"], dmin=c["dmin"],
                            seed=seed)


def alloy_labels(cell, sp, pos):
    c = ALLOY
    return syn.lennard_jones(cell, sp, pos, c["eps"], c["lj_sigma"], c["rc"])


def alloy_sparse_choice(n_train, species_lists, per_species, seed):
    """Per training structure, the sorted atom indices chosen as sparse
    environments: per species, ``per_species`` draws without replacement
    from the pool of all training atoms of that species."""
    r = syn.rng(seed)
    chosen = [[] for _ in range(n_train)]
    S = max(int(max(s)) for s in species_lists) + 1
    for s in range(S):
        pool = [(t, a) for t in range(n_train)
                for a in np.nonzero(np.asarray(species_lists[t]) == s)[0]]
        k = min(per_species, len(pool))
        pick = r.choice(len(pool), size=k, replace=False)
        for q in pick:
            t, a = pool[q]
            chosen[t].append(int(a))
    return [sorted(c) for c in chosen]


def build_alloy_model(n_train=None, per_species=None, verbose=False):
    """Train the alloy model with flare_gb300 (GPU, FP64).  Returns
    (SparseGP, B2, NormalizedDotProduct)."""
    import flare_gb300 as fg
    c = ALLOY
    n_train = n_train or c["n_train"]
    per_species = per_species or c["sparse_per_species"]
    b2 = fg.B2("chebyshev", "quadratic", [0.0, c["rc"]], [],
               [2, c["n_max"], c["l_max"]])
    k = fg.NormalizedDotProduct(c["sigma"], c["power"])
    gp = fg.SparseGP([k], c["sigma_e_per_atom"] * c["n_atoms"], c["sigma_f"],
                     c["sigma_s"])
    data = [alloy_structure(c["train_seed0"] + t) for t in range(n_train)]
    sparse = alloy_sparse_choice(n_train, [d[1] for d in data], per_species,
                                 c["sparse_seed"])
    for t, (cell, sp, pos) in enumerate(data):
        st = fg.Structure(cell, sp, pos, c["rc"], [b2])
        E, F, _ = alloy_labels(cell, sp, pos)
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        gp.add_training_structure(st)
        gp.add_specific_environments(st, sparse[t])
        if verbose:
            print(f"  trained structure {t}: M = {gp.n_sparse}", flush=True)
    gp.update_matrices_QR()
    return gp, b2, k


# ``fcc1m``: 64x64x64 FCC cells (1,048,576 atoms, a = 4.05 A) with thermal
# Gaussian displacements sigma = 0.08 A (seed 3000); B2 n_max = 10, l_max = 6,
# rc = 5.0 A; model: 4,000 sparse environments from 16 seeded 256-atom FCC
# structures at sigma = 0.08 (seeds 3001-3016), LJ energy and force labels.
# ``fcc256``: the reference's small, CPU-runnable case: 4 x 4 x 4 FCC cells
# (256 atoms, a = 4.05 A), Gaussian displacements sigma 0.05 A; B2
# chebyshev/quadratic [1, 8, 3], rc 5.0 A; NormalizedDotProduct sigma 2,
# power 2; 20 training cells (seeds 1000-1019) with truncated LJ energies and
# forces (eps 0.4 eV, sigma 2.6 A); 200 sparse environments drawn without
# replacement from the 20 x 256 pool (seed 1200); noise sigma_E 1e-3
# eV/atom (0.256 eV per structure), sigma_F 0.05 eV/A, no stress labels;
# test cells from seeds 1100, 1101, ...
FCC256 = dict(n_cells=4, a=4.05, sigma_disp=0.05, rc=5.0, n_max=8, l_max=3,
              sigma=2.0, power=2, n_train=20, train_seed0=1000, n_sparse=200,
              sparse_seed=1200, test_seed0=1100, sigma_e=0.256, sigma_f=0.05,
              sigma_s=1.0)


def fcc256_structure(seed):
    c = FCC256
    return syn.fcc_al(n_cells=c["n_cells"], a=c["a"], sigma=c["sigma_disp"],
                      seed=seed)


def fcc256_sparse_choice():
    c = FCC256
    chosen = syn.rng(c["sparse_seed"]).choice(c["n_train"] * 256,
                                              size=c["n_sparse"], replace=False)
    return [sorted(int(q) - 256 * t for q in chosen if q // 256 == t)
            for t in range(c["n_train"])]


def build_fcc256_model():
    """Train the fcc256 model on the GPU (FP64)."""
    import flare_gb300 as fg
    c = FCC256
    b2 = fg.B2("chebyshev", "quadratic", [0.0, c["rc"]], [],
               [1, c["n_max"], c["l_max"]])
    k = fg.NormalizedDotProduct(c["sigma"], c["power"])
    gp = fg.SparseGP([k], c["sigma_e"], c["sigma_f"], c["sigma_s"])
    sparse = fcc256_sparse_choice()
    for t in range(c["n_train"]):
        cell, sp, pos = fcc256_structure(c["train_seed0"] + t)
        st = fg.Structure(cell, sp, pos, c["rc"], [b2])
        E, F, _ = syn.lennard_jones(cell, sp, pos, [0.4], [2.6], c["rc"])
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        gp.add_training_structure(st)
        gp.add_specific_environments(st, sparse[t])
    gp.update_matrices_QR()
    return gp, b2, k


FCC1M = dict(n_cells=64, a=4.05, sigma_disp=0.08, seed=3000, rc=5.0, n_max=10,
             l_max=6, sigma=2.0, power=2, n_train=16, train_seed0=3001,
             n_sparse=4000, sparse_seed=3200, sigma_e_per_atom=1e-3,
             sigma_f=0.05, sigma_s=1.0)


def build_fcc_model(n_train=None, n_sparse=None):
    """Train the large-structure model on the GPU (FP64)."""
    import flare_gb300 as fg
    c = FCC1M
    n_train = n_train or c["n_train"]
    n_sparse = n_sparse or c["n_sparse"]
    b2 = fg.B2("chebyshev", "quadratic", [0.0, c["rc"]], [],
               [1, c["n_max"], c["l_max"]])
    k = fg.NormalizedDotProduct(c["sigma"], c["power"])
    gp = fg.SparseGP([k], c["sigma_e_per_atom"] * 256, c["sigma_f"],
                     c["sigma_s"])
    r = syn.rng(c["sparse_seed"])
    chosen = r.choice(n_train * 256, size=min(n_sparse, n_train * 256),
                      replace=False)
    for t in range(n_train):
        cell, sp, pos = syn.fcc_al(n_cells=4, a=c["a"], sigma=c["sigma_disp"],
                                   seed=c["train_seed0"] + t)
        st = fg.Structure(cell, sp, pos, c["rc"], [b2])
        E, F, _ = syn.lennard_jones(cell, sp, pos, [0.4], [2.6], c["rc"])
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        gp.add_training_structure(st)
        atoms = sorted(int(q) - 256 * t for q in chosen if q // 256 == t)
        gp.add_specific_environments(st, atoms)
    gp.update_matrices_QR()
    return gp, b2, k


def fcc_structure(n_cells=None, seed=None):
    c = FCC1M
    return syn.fcc_al(n_cells=n_cells or c["n_cells"], a=c["a"],
                      sigma=c["sigma_disp"], seed=seed or c["seed"])


# ``md3``: an ensemble of 2,000-atom 3-species cubic cells at
# 0.06 atoms/A^3 (species fractions 0.5/0.3/0.2, masses 27/58/1 amu), filled
# by random sequential addition with a 1.8 A minimum distance (replica r:
# seed 5000 + r), Maxwell-Boltzmann velocities at 1,200 K (seed 5500 + r),
# velocity Verlet dt = 1 fs; atoms flagged when their local std (divided by
# sigma, as the reference calculator reports it) exceeds 0.05.
# Model: B2 chebyshev/quadratic [3, 8, 4], rc 5.5 A (n_d = 1,500);
# NormalizedDotProduct sigma 2, power 2; 8,000 sparse environments = every
# atom of 4 training cells (seeds 5600-5603) labelled by truncated LJ energies
# and forces (eps 0.4/0.25/0.1 eV, sigma 1.8/1.7/1.5 A, Lorentz-Berthelot
# mixing: the 1.8 A minimum distance of the cells sits at or beyond sigma, so
# the replicas start near the potential's repulsive edge instead of high up
# its wall); noise sigma_E 1e-3 eV/atom, sigma_F 0.05 eV/A.  The sparse set then
# grows by the 256 most uncertain environments of the ensemble and is
# re-solved in FP64.
MD3 = dict(n_atoms=2000, density=0.06, fractions=(0.5, 0.3, 0.2), dmin=1.8,
           masses=(27.0, 58.0, 1.0), temperature=1200.0, dt=1.0,
           std_threshold=0.05, n_replicas=256, replica_seed0=5000,
           velocity_seed0=5500, rc=5.5, n_max=8, l_max=4, sigma=2.0, power=2,
           n_train=4, train_seed0=5600, eps=(0.4, 0.25, 0.1),
           lj_sigma=(1.8, 1.7, 1.5), sigma_e_per_atom=1e-3, sigma_f=0.05,
           sigma_s=1.0, n_grow=256)


def md_cell(seed):
    c = MD3
    return syn.rsa_alloy(c["n_atoms"], density=c["density"],
                         fractions=c["fractions"], dmin=c["dmin"], seed=seed)


def md_replicas(n, processes=8):
    """Replica cells ``md_cell(replica_seed0 + r)``, r < n, generated by a
    pool of spawned processes (safe after CUDA is initialised)."""
    import multiprocessing as mp
    seeds = [MD3["replica_seed0"] + r for r in range(n)]
    if n <= 4 or processes <= 1:
        return [md_cell(s) for s in seeds]
    with mp.get_context("spawn").Pool(min(processes, n)) as pool:
        return pool.map(md_cell, seeds)


def build_md_model(n_train=None):
    """Train the 3-species ensemble model on the GPU (FP64); every atom of
    the training cells is a sparse environment."""
    import flare_gb300 as fg
    c = MD3
    n_train = n_train or c["n_train"]
    b2 = fg.B2("chebyshev", "quadratic", [0.0, c["rc"]], [],
               [3, c["n_max"], c["l_max"]])
    k = fg.NormalizedDotProduct(c["sigma"], c["power"])
    gp = fg.SparseGP([k], c["sigma_e_per_atom"] * c["n_atoms"], c["sigma_f"],
                     c["sigma_s"])
    for t in range(n_train):
        cell, sp, pos = md_cell(c["train_seed0"] + t)
        st = fg.Structure(cell, sp, pos, c["rc"], [b2])
        E, F, _ = syn.lennard_jones(cell, sp, pos, c["eps"], c["lj_sigma"],
                                    c["rc"])
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        gp.add_training_structure(st)
        gp.add_specific_environments(st, list(range(len(sp))))
    gp.update_matrices_QR()
    return gp, b2, k


# ``serve3``: prediction requests of uneven size and species mix.
# Request q (seed 4000 + q): N = floor(exp(U[ln 32, ln 4096])) atoms, a
# uniformly drawn number (1-3) of the 3 species with fractions uniform on the
# simplex, density U[0.05, 0.09] atoms/A^3, random sequential addition with a
# 1.8 A minimum distance.  Model: the alloy1000 descriptor and kernel
# settings with 3 species (B2 [3, 8, 4], rc 5.5 A, n_d 1,500), 1,000 sparse
# environments per species drawn (seed 4300) from 10 training cells of 1,000
# atoms (seeds 4200-4209, species 1/3 each, density 0.06) with the md3 LJ
# labels.
SERVE3 = dict(n_requests=4096, seed0=4000, n_min=32, n_max_atoms=4096,
              density=(0.05, 0.09), dmin=1.8, rc=5.5, n_max=8, l_max=4,
              sigma=2.0, power=2, n_train=10, train_atoms=1000,
              train_seed0=4200, sparse_per_species=1000, sparse_seed=4300,
              sigma_e_per_atom=1e-3, sigma_f=0.05, sigma_s=1.0)


def serve_request(q):
    """Request q of the serving stream: (cell, species, positions)."""
    c = SERVE3
    r = syn.rng(c["seed0"] + q)
    n = int(np.floor(np.exp(r.uniform(np.log(c["n_min"]),
                                      np.log(c["n_max_atoms"])))))
    k = int(r.integers(1, 4))
    present = r.choice(3, size=k, replace=False)
    fr = np.zeros(3)
    fr[present] = r.dirichlet(np.ones(k))
    dens = float(r.uniform(*c["density"]))
    return syn.rsa_alloy(n, density=dens, fractions=fr, dmin=c["dmin"],
                         seed=c["seed0"] + 100000 + q)


def serve_requests(n, processes=16):
    """The first n requests, generated by spawned worker processes."""
    import multiprocessing as mp
    if n <= 8 or processes <= 1:
        return [serve_request(q) for q in range(n)]
    with mp.get_context("spawn").Pool(processes) as pool:
        return pool.map(serve_request, range(n), chunksize=16)


def build_serve_model():
    """Train the 3-species serving model on the GPU (FP64)."""
    import flare_gb300 as fg
    c, m = SERVE3, MD3
    b2 = fg.B2("chebyshev", "quadratic", [0.0, c["rc"]], [],
               [3, c["n_max"], c["l_max"]])
    k = fg.NormalizedDotProduct(c["sigma"], c["power"])
    gp = fg.SparseGP([k], c["sigma_e_per_atom"] * c["train_atoms"],
                     c["sigma_f"], c["sigma_s"])
    data = [syn.rsa_alloy(c["train_atoms"], density=0.06,
                          fractions=(1 / 3, 1 / 3, 1 / 3), dmin=c["dmin"],
                          seed=c["train_seed0"] + t)
            for t in range(c["n_train"])]
    sparse = alloy_sparse_choice(c["n_train"], [d[1] for d in data],
                                 c["sparse_per_species"], c["sparse_seed"])
    for t, (cell, sp, pos) in enumerate(data):
        st = fg.Structure(cell, sp, pos, c["rc"], [b2])
        E, F, _ = syn.lennard_jones(cell, sp, pos, m["eps"], m["lj_sigma"],
                                    c["rc"])
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        gp.add_training_structure(st)
        gp.add_specific_environments(st, sparse[t])
    gp.update_matrices_QR()
    return gp, b2, k
