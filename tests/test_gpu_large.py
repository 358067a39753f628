"""GPU: the large-structure path — a 131,072-atom FCC cell (32^3 cells) on
the fcc1m model (B2 n_max 10, l_max 6, 4,000 sparse environments): forces
and virial from the reverse-mode adjoint against finite differences of the
FP64 energy (h = 1e-4 A) over 64 random atoms, by directional derivatives."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fcc_model():
    from flare_gb300 import workloads as wl
    gp, b2, k = wl.build_fcc_model(n_train=6, n_sparse=1200)
    return gp, b2


def _predict(gp, b2, cell, sp, pos, precision):
    import flare_gb300 as fg
    return gp.predict_batch([fg.Structure(cell, sp, pos, 5.0, [b2])], want=7,
                            precision=precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_directional_finite_differences(fcc_model, precision):
    from flare_gb300 import workloads as wl
    gp, b2 = fcc_model
    # the mixed path's kernel GEMM at 9 slices: the energy then resolves
    # h F (its rounding at 7 slices, summed over the atoms near the moved
    # ones, moves a central difference by ~1e-3 eV/A); the forces are the
    # mixed path's own (FP32-level fold GEMM, FP32 adjoint)
    gp.set_slices(9, 0)
    cell, sp, pos = wl.fcc_structure(n_cells=32, seed=3100)
    r = _predict(gp, b2, cell, sp, pos, precision)
    F = r["forces"]
    rng = np.random.Generator(np.random.PCG64(3100))
    atoms = rng.choice(len(sp), size=64, replace=False)
    h = 1e-4
    for trial in range(2):
        d = np.zeros_like(pos)
        d[atoms] = rng.normal(size=(64, 3))
        d /= np.linalg.norm(d[atoms], axis=1).max()
        ep = _predict(gp, b2, cell, sp, pos + h * d, precision)["energy"][0]
        em = _predict(gp, b2, cell, sp, pos - h * d, precision)["energy"][0]
        fd = -(ep - em) / (2 * h)
        an = float(np.sum(F * d))
        # FP64 energy of 131k atoms resolves h*F to ~1e-8 eV
        assert abs(fd - an) < 1e-4 * max(1.0, abs(an)), (fd, an)
    # virial xx by a homogeneous strain of cell and positions
    eps = np.eye(3)
    eps[0, 0] += h
    ep = _predict(gp, b2, cell @ eps, sp, pos @ eps, precision)["energy"][0]
    eps[0, 0] -= 2 * h
    em = _predict(gp, b2, cell @ eps, sp, pos @ eps, precision)["energy"][0]
    vol = abs(np.linalg.det(cell))
    fd_sxx = -(ep - em) / (2 * h) / vol
    assert abs(fd_sxx - r["stress"][0][0]) < 1e-6 + 1e-4 * abs(fd_sxx)
