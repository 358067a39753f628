"""CPU: the seeded synthetic inputs of the benchmarks and tests
(flare_gb300/synthetic.py, flare_gb300/workloads.py) have the stated
shapes, densities, minimum distances and species mixes, repeat for a
seed, and their Lennard-Jones labels are consistent: forces are minus the
energy gradient, and the stress is -(1/V) dE/d(strain) in flare order
(xx, xy, xz, yy, yz, zz)."""
import numpy as np
import pytest

from flare_gb300 import synthetic as syn
from flare_gb300 import workloads as wl


def _min_periodic_distance(cell, pos):
    L = np.diag(cell)
    d = pos[:, None, :] - pos[None, :, :]
    d -= L * np.round(d / L)
    r2 = np.einsum("ijk,ijk->ij", d, d)
    np.fill_diagonal(r2, np.inf)
    return np.sqrt(r2.min())


def test_fcc_shape_and_seed():
    cell, sp, pos = syn.fcc_al(n_cells=3, a=4.05, sigma=0.05, seed=7)
    assert pos.shape == (4 * 27, 3) and (sp == 0).all()
    assert np.allclose(cell, np.eye(3) * 12.15)
    _, _, again = syn.fcc_al(n_cells=3, a=4.05, sigma=0.05, seed=7)
    assert np.array_equal(pos, again)
    _, _, ideal = syn.fcc_al(n_cells=3, a=4.05, sigma=0.0, seed=7)
    disp = pos - ideal
    assert 0.03 < disp.std() < 0.07


@pytest.mark.parametrize("gen", [syn.random_alloy, syn.rsa_alloy])
def test_alloy_density_distance_species(gen):
    n, dens, dmin = 400, 0.06, 1.8
    cell, sp, pos = gen(n, density=dens, fractions=(0.7, 0.3), dmin=dmin,
                        seed=11)
    assert pos.shape == (n, 3) and sp.shape == (n,)
    assert np.linalg.det(cell) == pytest.approx(n / dens, rel=1e-12)
    assert ((pos >= 0) & (pos <= cell[0, 0])).all()
    assert _min_periodic_distance(cell, pos) >= dmin * (1 - 1e-12)
    assert set(np.unique(sp)) <= {0, 1}
    assert 0.6 < np.mean(sp == 0) < 0.8
    _, sp2, pos2 = gen(n, density=dens, fractions=(0.7, 0.3), dmin=dmin,
                       seed=11)
    assert np.array_equal(pos, pos2) and np.array_equal(sp, sp2)


def test_alloy1000_structure():
    cell, sp, pos = wl.alloy_structure(2100)
    assert pos.shape == (1000, 3)
    assert np.linalg.det(cell) == pytest.approx(1000 / 0.06, rel=1e-12)
    assert _min_periodic_distance(cell, pos) >= 1.8 * (1 - 1e-12)


def test_serving_requests_in_range():
    c = wl.SERVE3
    for q in range(6):
        cell, sp, pos = wl.serve_request(q)
        n = len(pos)
        assert c["n_min"] <= n <= c["n_max_atoms"]
        dens = n / np.linalg.det(cell)
        assert c["density"][0] * (1 - 1e-9) <= dens <= c["density"][1] * (1 + 1e-9)
        assert 1 <= len(np.unique(sp)) <= 3 and sp.max() < 3


def _lj_cell():
    cell, _, pos = syn.fcc_al(n_cells=2, a=4.05, sigma=0.12, seed=3)
    sp = np.array([0, 1] * (len(pos) // 2))
    return cell, sp, pos


EPS, SIG, RC = (0.4, 0.25), (2.6, 2.3), 5.5


def test_lj_forces_are_minus_gradient():
    cell, sp, pos = _lj_cell()
    _, f, _ = syn.lennard_jones(cell, sp, pos, EPS, SIG, RC)
    h = 1e-5
    for a in (0, 5, 17):
        for k in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[a, k] += h
            p2[a, k] -= h
            e1 = syn.lennard_jones(cell, sp, p1, EPS, SIG, RC)[0]
            e2 = syn.lennard_jones(cell, sp, p2, EPS, SIG, RC)[0]
            assert f[a, k] == pytest.approx(-(e1 - e2) / (2 * h), abs=1e-6)
    assert np.allclose(f.sum(axis=0), 0.0, atol=1e-10)


def test_lj_stress_is_strain_derivative():
    cell, sp, pos = _lj_cell()
    _, _, s = syn.lennard_jones(cell, sp, pos, EPS, SIG, RC)
    vol = abs(np.linalg.det(cell))
    h = 1e-6
    order = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for q, (a, b) in enumerate(order):
        eps = np.zeros((3, 3))
        eps[a, b] = eps[b, a] = h     # symmetric strain
        es = []
        for sgn in (1, -1):
            m = np.eye(3) + sgn * eps
            es.append(syn.lennard_jones(cell @ m, sp, pos @ m, EPS, SIG, RC)[0])
        de = (es[0] - es[1]) / (2 * h)
        if a != b:
            de /= 2   # both off-diagonal entries moved
        assert s[q] == pytest.approx(-de / vol, abs=1e-7)
