"""GPU: SGP_Wrapper / SGP_Calculator (flare/bffs/sgp/sparse_gp.py and
calculator.py) against the oracle, and the reference's JSON round-trip
checks (tests/test_sparse_gp.py:23-135)."""
import os

import numpy as np
import pytest

import oracle
from helpers import b2_args, lj_labels, random_atoms

pytestmark = pytest.mark.gpu


class Atoms:
    def __init__(self, cell, numbers, positions):
        self.cell = cell
        self.numbers = numbers
        self.positions = positions


def make_wrapper(variance_type="local", multicut=False, power=2):
    import flare_gb300 as fg
    S = 2
    cutoffs = (5.0 * np.ones((S, S)) + np.eye(S) - 1) if multicut else None
    b2a = b2_args(S, 3, 2, 5.0, cutoffs=cutoffs)
    calc = fg.B2(*b2a[:5], cutoffs=cutoffs)
    k = fg.NormalizedDotProduct(1.3, power)
    sae = {0: 0.37, 1: -0.21}
    w = fg.SGP_Wrapper([k], [calc], 5.0, 0.4, 0.3, 0.5, {6: 0, 8: 1},
                       variance_type=variance_type, single_atom_energies=sae)
    return w, b2a, sae


def train(w, sae, seeds=(1, 2), sizes=(5, 6)):
    data = []
    for seed, size in zip(seeds, sizes):
        cell, sp, pos = random_atoms(seed=seed)
        E, F, St = lj_labels(cell, sp, pos, 2)
        numbers = np.where(sp == 0, 6, 8)
        r = np.random.Generator(np.random.PCG64(seed + 100))
        custom = sorted(r.choice(len(sp), size=size, replace=False).tolist())
        w.update_db(Atoms(cell, numbers, pos), F, custom_range=custom,
                    energy=E, stress=St, mode="specific",
                    rel_e_noise=0.5, rel_f_noise=0.8, rel_s_noise=0.9)
        data.append((cell, sp, pos, E, F, St, custom))
    return data


def oracle_twin(w, b2a, sae, data):
    k = w.sparse_gp.kernels[0]
    ogp = oracle.SparseGP([oracle.NormalizedDotProduct(k.sigma, k.power)],
                          w.sparse_gp.energy_noise, w.sparse_gp.force_noise,
                          w.sparse_gp.stress_noise)
    ob2 = oracle.B2Settings(*b2a)
    for cell, sp, pos, E, F, St, custom in data:
        st = oracle.Structure(cell, sp, pos, 5.0, [ob2])
        st.energy = np.array([E - sum(sae[s] for s in sp)])
        st.forces = F.reshape(-1)
        st.stresses = St
        ogp.add_training_structure(st, [-1], 0.5, 0.8, 0.9)
        ogp.add_specific_environments(st, custom)
    ogp.update_matrices_QR()
    return ogp, ob2


@pytest.mark.parametrize("vt", ["local", "SOR", "DTC"])
@pytest.mark.parametrize("multicut", [False, True])
def test_calculator_matches_oracle(vt, multicut):
    import flare_gb300 as fg
    w, b2a, sae = make_wrapper(vt, multicut)
    data = train(w, sae)
    ogp, ob2 = oracle_twin(w, b2a, sae, data)
    cell, sp, pos = random_atoms(seed=42)
    calc = fg.SGP_Calculator(w)
    calc.calculate(Atoms(cell, np.where(sp == 0, 6, 8), pos))
    st = oracle.Structure(cell, sp, pos, 5.0, [ob2])
    if vt == "local":
        ogp.predict_local_uncertainties(st)
    elif vt == "SOR":
        ogp.predict_SOR(st)
    else:
        ogp.predict_DTC(st)
    ref = oracle.calculator_results(st, vt, w.hyps[0], sae)
    scale = max(1.0, abs(ref["energy"]))
    assert abs(calc.results["energy"] - ref["energy"]) < 1e-8 * scale
    np.testing.assert_allclose(calc.results["forces"], ref["forces"],
                               atol=1e-7 * max(1, np.abs(ref["forces"]).max()))
    np.testing.assert_allclose(calc.results["stress"], ref["stress"],
                               atol=1e-8 * max(1, np.abs(ref["stress"]).max()))
    np.testing.assert_allclose(calc.results["stds"], ref["stds"], rtol=1e-5,
                               atol=1e-6)


def test_update_db_sizes():
    """test_sparse_gp.py:23-44."""
    import flare_gb300 as fg
    w, b2a, sae = make_wrapper()
    cell, sp, pos = random_atoms(seed=7)
    E, F, St = lj_labels(cell, sp, pos, 2)
    w.update_db(Atoms(cell, np.where(sp == 0, 6, 8), pos), F, [1, 2, 3], E, St,
                mode="specific")
    assert w.sparse_gp.Kuu.shape[0] == 3
    assert w.sparse_gp.Kuf.shape[1] == 1 + len(sp) * 3 + 6


def test_write_model_reload_forces(tmp_path):
    """test_sparse_gp.py:105-135: a reconstructed calculator predicts the
    same forces (max abs difference < 1e-8)."""
    import flare_gb300 as fg
    w, b2a, sae = make_wrapper("local")
    train(w, sae)
    calc = fg.SGP_Calculator(w)
    cell, sp, pos = random_atoms(seed=31)
    at = Atoms(cell, np.where(sp == 0, 6, 8), pos)
    calc.calculate(at)
    f1 = calc.results["forces"].copy()
    name = os.path.join(str(tmp_path), "sgp_calc.json")
    calc.write_model(name)
    calc2, _ = fg.SGP_Calculator.from_file(name)
    calc2.calculate(at)
    assert np.max(np.abs(f1 - calc2.results["forces"])) < 1e-8
    assert len(calc2.gp_model) == len(w)
    np.testing.assert_allclose(calc2.gp_model.hyps, w.hyps)


def test_other_sparse_modes():
    """update_db modes all / random / uncertain grow the sparse set."""
    import flare_gb300 as fg
    w, b2a, sae = make_wrapper("local")
    cell, sp, pos = random_atoms(seed=8)
    E, F, St = lj_labels(cell, sp, pos, 2)
    at = Atoms(cell, np.where(sp == 0, 6, 8), pos)
    w.update_db(at, F, [], E, St, mode="all")
    assert w.sparse_gp.n_sparse == len(sp)
    cell, sp, pos = random_atoms(seed=9)
    E, F, St = lj_labels(cell, sp, pos, 2)
    at = Atoms(cell, np.where(sp == 0, 6, 8), pos)
    w.update_db(at, F, [3], E, St, mode="random")
    assert w.sparse_gp.n_sparse == 2 * len(sp) - len(sp) + 3
    cell, sp, pos = random_atoms(seed=10)
    E, F, St = lj_labels(cell, sp, pos, 2)
    at = Atoms(cell, np.where(sp == 0, 6, 8), pos)
    w.update_db(at, F, [4], E, St, mode="uncertain")
    assert w.sparse_gp.n_sparse == len(sp) + 3 + 4
