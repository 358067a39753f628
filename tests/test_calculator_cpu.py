"""CPU: SGP_Calculator's post-processing of a prediction
(flare/bffs/sgp/calculator.py:57-122, sort_variances at :188-206), driven
by stand-in model and structure objects so that no GPU call is made:
energy with single-atom energies, forces, the flare -> ASE stress order
and sign, and the signed standard deviations of the SOR/DTC and local
variance types (local: species-sorted variances back in atom order,
divided by |sigma|)."""
from types import SimpleNamespace

import numpy as np
import pytest

from flare_gb300.calculator import SGP_Calculator, sort_variances

N = 5
SPECIES = [1, 0, 1, 0, 0]
# atoms of species 0 are 1, 3, 4; of species 1, 0 and 2
ATOM_INDICES = [[1, 3, 4], [0, 2]]


class _FakeSparseGP:
    def __init__(self):
        self.calls = []

    def predict_SOR(self, s):
        self.calls.append("SOR")

    def predict_DTC(self, s):
        self.calls.append("DTC")

    def predict_local_uncertainties(self, s):
        self.calls.append("local")


def _structure():
    mean = np.arange(1 + 3 * N + 6, dtype=np.float64) * 0.5 - 3.0
    var_efs = np.linspace(-0.3, 2.5, 1 + 3 * N + 6)
    # species-sorted local variances: atoms 1, 3, 4 (species 0), then 0, 2
    local = np.array([4.0, -0.25, 0.0, 9.0, 1e-6])
    return SimpleNamespace(
        noa=N, species=SPECIES, mean_efs=mean, variance_efs=var_efs,
        local_uncertainties=[local],
        descriptors=[SimpleNamespace(n_types=2, atom_indices=ATOM_INDICES)])


def _calculator(vt, single=None, sigma=-2.0):
    gp = SimpleNamespace(variance_type=vt, sparse_gp=_FakeSparseGP(),
                         single_atom_energies=single,
                         hyps=np.array([sigma, 0.1, 0.05, 0.01]))
    return SGP_Calculator(gp), gp


def test_sort_variances_to_atom_order():
    s = _structure()
    out = sort_variances(s, s.local_uncertainties[0])
    # atom a gets the value at its position in the species-sorted list
    assert out.tolist() == [9.0, 4.0, 1e-6, -0.25, 0.0]


@pytest.mark.parametrize("vt", ["SOR", "DTC", "local"])
def test_calls_the_variance_types_prediction(vt):
    calc, gp = _calculator(vt)
    calc.predict_on_structure(_structure())
    assert gp.sparse_gp.calls == [vt]


def test_energy_forces_stress():
    s = _structure()
    calc, _ = _calculator("local", single={0: -1.5, 1: 0.25})
    calc.predict_on_structure(s)
    m = s.mean_efs
    # three atoms of species 0, two of species 1
    assert calc.results["energy"] == pytest.approx(m[0] + 3 * -1.5 + 2 * 0.25)
    assert np.array_equal(calc.results["forces"], m[1:-6].reshape(N, 3))
    xx, xy, xz, yy, yz, zz = m[-6:]   # flare order
    # ASE order (xx, yy, zz, yz, xz, xy), sign flipped
    assert np.array_equal(calc.results["stress"],
                          -np.array([xx, yy, zz, yz, xz, xy]))


def test_energy_without_single_atom_energies():
    s = _structure()
    calc, _ = _calculator("SOR")
    calc.predict_on_structure(s)
    assert calc.results["energy"] == s.mean_efs[0]


@pytest.mark.parametrize("vt", ["SOR", "DTC"])
def test_force_stds_signed(vt):
    s = _structure()
    calc, _ = _calculator(vt)
    calc.predict_on_structure(s)
    v = s.variance_efs[1:-6]
    want = np.array([np.sqrt(x) if x > 0 else -np.sqrt(-x) for x in v])
    assert calc.results["stds"].shape == (N, 3)
    assert np.array_equal(calc.results["stds"].ravel(), want)
    assert (calc.results["stds"].ravel()[v < 0] < 0).all()


def test_local_stds_in_atom_order_over_sigma():
    s = _structure()
    calc, _ = _calculator("local", sigma=-2.0)
    calc.predict_on_structure(s)
    stds = calc.results["stds"]
    assert stds.shape == (N, 3)
    # atom order: variances 9, 4, 1e-6, -0.25, 0; divided by |sigma| = 2
    want = np.array([3.0, 2.0, 1e-3, -0.5, 0.0]) / 2.0
    assert np.allclose(stds[:, 0], want, rtol=1e-15, atol=0)
    assert stds[3, 0] < 0 and stds[4, 0] == 0.0
    assert not stds[:, 1:].any()
