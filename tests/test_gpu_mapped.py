"""GPU: mapped models — the lmp.flare mapping coefficients against the
oracle's restatement of compute_map_coeff_pow1/pow2 and of the file writer;
evaluation from the file (pair style flare arithmetic) against the sparse
GP it came from; the variance map and the L_inverse / sparse-descriptor
files against the GP's local std."""
import numpy as np
import pytest

import oracle
from helpers import c1_model, small_two_species, to_gpu_sgp
from flare_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _items(n=3, seed=1500):
    return [syn.fcc_al(seed=seed + k) for k in range(n)]


def _strucs(calc, items, cutoff=5.0):
    import flare_gb300 as fg
    return [fg.Structure(c, s, p, cutoff, [calc]) for c, s, p in items]


@pytest.fixture(scope="module", params=[2, 1])
def model(request):
    ogp, b2a = c1_model(n_train=8, n_sparse=120, power=request.param)
    gp, calc = to_gpu_sgp(ogp, b2a)
    return request.param, ogp, gp, calc


def _abs_bound(ogp):
    """Per coefficient, the sum of the magnitudes of its terms
    sig^2 |alpha_j| |p_k| (|p_l|): FP64 sums in another order agree within
    a few n eps times it."""
    k, cd = ogp.kernels[0], ogp.sparse_descriptors[0]
    rows = []
    for s in range(cd.n_types):
        c = cd.cumulative_type_count[s]
        n = cd.n_clusters_by_type[s]
        P = np.abs(cd.descriptors[s] / cd.descriptor_norms[s][:, None])
        a = np.abs(ogp.alpha[c:c + n])
        if k.power == 1:
            rows.append(k.sigma ** 2 * (a @ P))
        else:
            B = k.sigma ** 2 * (P.T * a) @ P
            iu = np.triu_indices(B.shape[0])
            rows.append(B[iu] * np.where(iu[0] == iu[1], 1.0, 2.0))
    return np.stack(rows), cd.n_clusters


def test_coefficients_match_oracle(model, tmp_path):
    from flare_gb300 import mapped
    power, ogp, gp, calc = model
    f = tmp_path / "lmp.flare"
    ours = gp.write_mapping_coefficients(str(f), "tester", 0)
    ref = oracle.mapping_coefficients(ogp)
    bound, n = _abs_bound(ogp)
    err = np.abs(ours - ref)
    assert np.all(err <= 4 * n * 2.0 ** -53 * bound + 1e-300), \
        float(np.max(err / (bound + 1e-300)))
    info = mapped.read_mapping_file(str(f))
    assert info["power"] == power and info["kernel"] == "NormalizedDotProduct"
    assert info["descriptor_settings"] == list(calc.descriptor_settings)
    # the file holds the same numbers (16 significant digits)
    back = info["beta"]
    if power == 2:
        iu = np.triu_indices(back.shape[1])
        fac = np.where(iu[0] == iu[1], 1.0, 2.0)
        back = np.stack([b[iu] * fac for b in back])
    np.testing.assert_allclose(back, ours, rtol=1e-15, atol=0)


def test_file_text_matches_oracle_writer(model, tmp_path):
    power, ogp, gp, calc = model
    f = tmp_path / "lmp.flare"
    ours = gp.write_mapping_coefficients(str(f), "tester", 0)
    text = f.read_text()
    date = text.splitlines()[0][len("DATE: "):].split(" CONTRIBUTOR:")[0]
    ref = oracle.write_mapping_text(ours, power, calc.descriptor_settings,
                                    calc.radial_basis, calc.cutoff_function,
                                    calc.cutoffs, "tester", date)
    assert text == ref


def test_mapped_potential_matches_gp(model, tmp_path):
    """E_i = d^T beta d (power 2) is the GP mean folded into beta: the
    mapped energies, forces and stresses equal the FP64 GP predictions."""
    from flare_gb300.mapped import MappedPotential
    power, ogp, gp, calc = model
    f = tmp_path / "lmp.flare"
    gp.write_mapping_coefficients(str(f), "tester", 0)
    pot = MappedPotential(str(f))
    items = _items()
    a = gp.predict_batch(_strucs(calc, items), precision="fp64")
    b = pot.predict(_strucs(pot.b2, items))
    E = np.abs(a["energy"]).max()
    np.testing.assert_allclose(b["energy"], a["energy"], rtol=0,
                               atol=1e-10 * max(E, 1.0))
    np.testing.assert_allclose(b["forces"], a["forces"], rtol=0, atol=1e-8)
    np.testing.assert_allclose(b["stress"], a["stress"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(b["atom_energies"].reshape(3, -1).sum(1),
                               b["energy"], rtol=1e-12)


def test_mapped_energy_matches_oracle_formula(model, tmp_path):
    """Per-atom energies against compute_energy_and_u on the oracle's B2."""
    from flare_gb300.mapped import MappedPotential, read_mapping_file
    power, ogp, gp, calc = model
    f = tmp_path / "lmp.flare"
    gp.write_mapping_coefficients(str(f), "tester", 0)
    pot = MappedPotential(str(f))
    cell, sp, pos = _items(1, seed=1600)[0]
    r = pot.predict(_strucs(pot.b2, [(cell, sp, pos)]))
    info = read_mapping_file(str(f))
    b2a = (calc.radial_basis, calc.cutoff_function, calc.radial_hyps,
           calc.cutoff_hyps, calc.descriptor_settings, calc.cutoffs)
    st = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    dv = st.descriptors[0]
    for s in range(dv.n_types):
        for row, atom in enumerate(dv.atom_indices[s]):
            e, _ = oracle.mapped_energy_and_w(dv.descriptors[s][row],
                                              info["beta"][s], power)
            assert abs(r["atom_energies"][atom] - e) <= 1e-10 * max(abs(e), 1)


def test_local_std_from_files_matches_gp(tmp_path):
    """compute flare/std/atom (non-mapped form) from the L_inverse and
    sparse-descriptor files equals the GP's local std, two species."""
    from flare_gb300.calculator import SGP_Calculator  # noqa: F401
    from flare_gb300.mapped import LocalStdFromFiles
    ogp, b2a = small_two_species(seed=3, n_train=3, power=2)
    gp, calc = to_gpu_sgp(ogp, b2a)
    gp.write_L_inverse(str(tmp_path / "L_inv"), "tester")
    gp.write_sparse_descriptors(str(tmp_path / "sparse"), "tester")
    std_files = LocalStdFromFiles(str(tmp_path / "L_inv"),
                                  str(tmp_path / "sparse"))
    from helpers import random_atoms
    items = [random_atoms(seed=40 + k) for k in range(3)]
    v = gp.predict_batch(_strucs(calc, items), precision="fp64")["local_var"]
    sig = abs(gp.kernels[0].sigma)
    want = np.sign(v) * np.sqrt(np.abs(v)) / sig
    got = std_files.std(_strucs(std_files.b2, items))
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-9)


def test_varmap_std_matches_gp_power1(tmp_path):
    """The variance map of a power-1 model reproduces its local std
    (1 - |Q^T d^|^2 = var / sigma^2 for Kuu = sigma^2 S S^T + jitter)."""
    from flare_gb300.mapped import MappedPotential
    ogp, b2a = c1_model(n_train=8, n_sparse=120, power=1)
    gp, calc = to_gpu_sgp(ogp, b2a)
    gp.write_mapping_coefficients(str(tmp_path / "lmp"), "tester", 0)
    Q = gp.write_varmap_coefficients(str(tmp_path / "var"), "tester", 0)
    ref = oracle.varmap_coefficients(ogp)
    # Householder Q: the same columns (LAPACK and cuSOLVER conventions)
    np.testing.assert_allclose(np.abs(Q), np.abs(ref), rtol=0, atol=1e-9)
    pot = MappedPotential(str(tmp_path / "lmp"), str(tmp_path / "var"))
    items = _items(2, seed=1700)
    v = gp.predict_batch(_strucs(calc, items), precision="fp64")["local_var"]
    sig = abs(gp.kernels[0].sigma)
    want = np.sign(v) * np.sqrt(np.abs(v)) / sig
    got = pot.predict(_strucs(pot.b2, items), std=True)["std"]
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-6)


def test_calculator_build_map(tmp_path, monkeypatch):
    import flare_gb300 as fg
    ogp, b2a = c1_model(n_train=8, n_sparse=120, power=2)
    gp, calc = to_gpu_sgp(ogp, b2a)
    w = fg.SGP_Wrapper([gp.kernels[0]], [calc], 5.0, gp.energy_noise,
                       gp.force_noise, gp.stress_noise, {13: 0},
                       variance_type="local")
    w.sparse_gp = gp
    c = fg.SGP_Calculator(w)
    monkeypatch.chdir(tmp_path)
    c.build_map("lmp.flare", "tester")
    for name in ("lmp.flare", "L_inv_lmp.flare", "sparse_desc_lmp.flare"):
        assert (tmp_path / name).stat().st_size > 0
