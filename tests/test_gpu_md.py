"""GPU: the device MD ensemble (fgb_md_*, flare_gb300.md.Ensemble) —
velocity Verlet against a host integration with the library's own forces,
replica independence (bitwise), exact flag counts, energy conservation of
order dt^2, and growing the sparse set from the most uncertain environments
followed by the FP64 re-solve."""
import numpy as np
import pytest

from helpers import c1_model, to_gpu_sgp
from flare_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

MASSES = (27.0, 58.0)


def gpu_model(n_train=2, n_atoms=60, S=2):
    """Small 2-species model trained on the GPU (so its sparse set can
    grow): every fourth atom of each training cell is a sparse env."""
    import flare_gb300 as fg
    b2 = fg.B2("chebyshev", "quadratic", [0.0, 5.0], [], [S, 4, 2])
    k = fg.NormalizedDotProduct(2.0, 2)
    gp = fg.SparseGP([k], 0.1, 0.05, 1.0)
    for t in range(n_train):
        cell, sp, pos = syn.random_alloy(n_atoms, density=0.06,
                                         fractions=(0.5, 0.5), seed=9000 + t)
        st = fg.Structure(cell, sp, pos, 5.0, [b2])
        E, F, _ = syn.lennard_jones(cell, sp, pos, [0.4, 0.25], [2.6, 2.3], 5.0)
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        gp.add_training_structure(st)
        gp.add_specific_environments(st, list(range(0, n_atoms, 4)))
    gp.update_matrices_QR()
    return gp, b2


def replicas(n, n_atoms=60, seed=9100):
    return [syn.random_alloy(n_atoms, density=0.06, fractions=(0.5, 0.5),
                             seed=seed + r) for r in range(n)]


def test_velocity_verlet_matches_host_integration():
    import flare_gb300 as fg
    from flare_gb300.md import Ensemble, KACCEL
    gp, b2 = gpu_model()
    reps = replicas(2)
    ens = Ensemble(gp, [b2], reps, MASSES, temperature=300.0, seed=1,
                   precision="fp64")
    s0 = ens.state()
    x = s0["positions"].copy()
    v = s0["velocities"].copy()
    f = s0["forces"].copy()
    inv_m = 1.0 / np.asarray(MASSES)[ens.species]
    dt = 1.0

    def forces(xx):
        strucs = [fg.Structure(c, sp, xx[r * 60:(r + 1) * 60], 5.0, [b2])
                  for r, (c, sp, _) in enumerate(reps)]
        return gp.predict_batch(strucs, precision="fp64")["forces"]

    for _ in range(3):
        v = v + f * inv_m[:, None] * KACCEL * (0.5 * dt)
        x = x + v * dt
        f = forces(x)
        v = v + f * inv_m[:, None] * KACCEL * (0.5 * dt)
    ens.step(3, dt=dt)
    s = ens.state()
    np.testing.assert_allclose(s["positions"], x, rtol=0, atol=1e-10)
    np.testing.assert_allclose(s["velocities"], v, rtol=0, atol=1e-10)
    np.testing.assert_allclose(s["forces"], f, rtol=0, atol=1e-8)


def test_replica_same_alone_and_in_ensemble():
    from flare_gb300.md import Ensemble, maxwell_boltzmann
    gp, b2 = gpu_model()
    reps = replicas(3)
    vels = [maxwell_boltzmann(sp, MASSES, 600.0, 40 + r)
            for r, (_, sp, _) in enumerate(reps)]
    big = Ensemble(gp, [b2], reps, MASSES, velocities=np.concatenate(vels))
    one = Ensemble(gp, [b2], reps[1:2], MASSES, velocities=vels[1])
    big.step(4)
    one.step(4)
    a, b = big.state(), one.state()
    np.testing.assert_array_equal(a["positions"][60:120], b["positions"])
    np.testing.assert_array_equal(a["velocities"][60:120], b["velocities"])
    np.testing.assert_array_equal(a["local_var"][60:120], b["local_var"])


def test_flag_counts():
    from flare_gb300.md import Ensemble
    gp, b2 = gpu_model()
    ens = Ensemble(gp, [b2], replicas(2), MASSES, temperature=300.0, seed=3)
    ens.step(5, dt=0.5, std_threshold=-1.0)   # every atom counts
    assert np.all(ens.state()["flagged"] == 5 * 60)
    ens.step(3, dt=0.5, std_threshold=1e9)    # none does
    assert np.all(ens.state()["flagged"] == 5 * 60)


def test_energy_conservation_order_dt2():
    """Smooth FCC model, 300 K, FP64 forces: the total-energy error after
    20 fs shrinks about four-fold when dt halves."""
    from flare_gb300.md import Ensemble, maxwell_boltzmann
    ogp, b2a = c1_model(n_train=8, n_sparse=120, power=2)
    gp, calc = to_gpu_sgp(ogp, b2a)
    reps = [syn.fcc_al(seed=1300 + r) for r in range(2)]
    vel = np.concatenate([maxwell_boltzmann(sp, (27.0,), 300.0, 60 + r)
                          for r, (_, sp, _) in enumerate(reps)])
    errs = []
    for dt, n in ((1.0, 20), (0.5, 40)):
        ens = Ensemble(gp, [calc], reps, (27.0,), velocities=vel,
                       precision="fp64")
        s0 = ens.state()
        ens.step(n, dt=dt)
        s = ens.state()
        errs.append(np.max(np.abs(s["energy"] + s["kinetic"] -
                                  s0["energy"] - s0["kinetic"])) / 256)
    assert errs[0] < 1e-3, errs
    assert errs[1] < 0.5 * errs[0] or errs[0] < 1e-9, errs


def test_grow_sparse_set_lowers_uncertainty():
    from flare_gb300.md import Ensemble
    gp, b2 = gpu_model()
    ens = Ensemble(gp, [b2], replicas(2), MASSES, temperature=600.0, seed=5)
    ens.step(2)
    picks = ens.uncertain_environments(6)
    std0 = ens.state()["std"]
    before = np.array([std0[r * 60 + a] for r, a in picks])
    m0 = gp.n_sparse
    info = ens.grow_sparse_set(6)
    assert gp.n_sparse == m0 + 6 and info["sparse_after"] == m0 + 6
    std1 = ens.state()["std"]
    after = np.array([std1[r * 60 + a] for r, a in picks])
    assert np.all(after < before), (before, after)
    ens.step(2)                                  # continues with the new model
    assert np.all(np.isfinite(ens.state()["positions"]))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_replayed_steps_equal_full_steps(precision):
    """Graph-replayed steps (fixed neighbour rebuild, no host sync) give the
    same trajectory, bit for bit, as full checked steps; a change of dt or
    threshold recaptures."""
    from flare_gb300.md import Ensemble, maxwell_boltzmann
    gp, b2 = gpu_model()
    reps = replicas(3)
    vel = np.concatenate([maxwell_boltzmann(sp, MASSES, 900.0, 70 + r)
                          for r, (_, sp, _) in enumerate(reps)])
    g = Ensemble(gp, [b2], reps, MASSES, velocities=vel, precision=precision)
    f = Ensemble(gp, [b2], reps, MASSES, velocities=vel, precision=precision,
                 graphs=False)
    for n, dt, th in ((61, 1.0, 0.05), (7, 0.5, 0.05), (5, 0.5, 0.01)):
        g.step(n, dt=dt, std_threshold=th)
        f.step(n, dt=dt, std_threshold=th)
    a, b = g.state(), f.state()
    for k in ("positions", "velocities", "forces", "local_var", "energy",
              "kinetic", "max_std", "flagged"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    sg, sf = g.stats(), f.stats()
    assert sg["replayed"] > 0 and sg["captures"] >= 3, sg
    assert sf == {"replayed": 0, "full": 73, "captures": 0, "rollbacks": 0}
    assert sg["replayed"] + sg["full"] == 73


def test_pair_capacity_overflow_rolls_back():
    """A pair capacity below the current pair count: every replayed chunk
    overflows, is rolled back to its snapshot and redone with full steps;
    the trajectory is unchanged."""
    from flare_gb300.md import Ensemble, maxwell_boltzmann
    gp, b2 = gpu_model()
    reps = replicas(2)
    vel = np.concatenate([maxwell_boltzmann(sp, MASSES, 600.0, 80 + r)
                          for r, (_, sp, _) in enumerate(reps)])
    g = Ensemble(gp, [b2], reps, MASSES, velocities=vel, pair_margin=-0.2)
    f = Ensemble(gp, [b2], reps, MASSES, velocities=vel, graphs=False)
    g.step(12, std_threshold=0.02)
    f.step(12, std_threshold=0.02)
    a, b = g.state(), f.state()
    for k in ("positions", "velocities", "forces", "local_var", "flagged"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    s = g.stats()
    assert s["rollbacks"] >= 1 and s["replayed"] == 0 and s["full"] == 12, s
    # a normal margin afterwards replays again
    g.set_graphs(True, 0.25)
    f.step(10)
    g.step(10)
    np.testing.assert_array_equal(g.state()["positions"],
                                  f.state()["positions"])
    assert g.stats()["replayed"] == 10
