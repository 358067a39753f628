"""GPU: mean energy, forces, stress and local variance against the FP64
oracle (sparse_gp.cpp:643-757 + calculator.py post-processing), on the
same trained weights."""
import numpy as np
import pytest

import oracle
from helpers import (b2_args, c1_model, random_atoms, small_two_species,
                     to_gpu_sgp)
from flare_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

# FP64 path: tolerances for FP64 arithmetic in a different summation order.
E_TOL = 1e-9      # eV (absolute, whole structure) scaled by |E| below
F_TOL = 1e-8      # eV/A
S_TOL = 1e-10     # eV/A^3
V_TOL = 1e-10     # variance (absolute)


def oracle_predict(ogp, b2a, cell, sp, pos, cutoff=5.0):
    st = oracle.Structure(cell, sp, pos, cutoff, [oracle.B2Settings(*b2a)])
    ogp.predict_local_uncertainties(st)
    m = st.mean_efs
    var = oracle.sort_variances(st, st.local_uncertainties[0])
    return m[0], m[1:-6].reshape(-1, 3), m[-6:], var


def gpu_predict(ggp, calc, structures_np, cutoff=5.0, precision="fp64"):
    import flare_gb300 as fg
    strucs = [fg.Structure(c, s, p, cutoff, [calc]) for c, s, p in structures_np]
    return ggp.predict_batch(strucs, precision=precision)


@pytest.mark.parametrize("power", [1, 2])
def test_small_two_species_fp64(power):
    ogp, b2a = small_two_species(seed=5, n_train=3, power=power)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    cell, sp, pos = random_atoms(seed=55)
    E, F, S, V = oracle_predict(ogp, b2a, cell, sp, pos)
    r = gpu_predict(ggp, calc, [(cell, sp, pos)])
    assert abs(r["energy"][0] - E) < E_TOL * max(1, abs(E))
    np.testing.assert_allclose(r["forces"], F, atol=F_TOL)
    np.testing.assert_allclose(r["stress"][0], S, atol=S_TOL)
    np.testing.assert_allclose(r["local_var"], V, atol=V_TOL)


def test_multicut_model_fp64():
    ogp, b2a = small_two_species(seed=6, n_train=2, multicut=True)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    cell, sp, pos = random_atoms(seed=66)
    E, F, S, V = oracle_predict(ogp, b2a, cell, sp, pos)
    r = gpu_predict(ggp, calc, [(cell, sp, pos)])
    assert abs(r["energy"][0] - E) < E_TOL * max(1, abs(E))
    np.testing.assert_allclose(r["forces"], F, atol=F_TOL)
    np.testing.assert_allclose(r["stress"][0], S, atol=S_TOL)
    np.testing.assert_allclose(r["local_var"], V, atol=V_TOL)


@pytest.fixture(scope="module")
def c1():
    ogp, b2a = c1_model()
    ggp, calc = to_gpu_sgp(ogp, b2a)
    return ogp, b2a, ggp, calc


def test_fcc256_fp64(c1):
    ogp, b2a, ggp, calc = c1
    cell, sp, pos = syn.fcc_al(seed=1100)
    E, F, S, V = oracle_predict(ogp, b2a, cell, sp, pos)
    r = gpu_predict(ggp, calc, [(cell, sp, pos)])
    # |alpha| ~ 1e4 makes the sum of kernel terms cancel; FP64 agreement
    # is limited by that cancellation (oracle vs long double: ~1e-9 eV).
    assert abs(r["energy"][0] - E) < 1e-7
    np.testing.assert_allclose(r["forces"], F, atol=1e-7)
    np.testing.assert_allclose(r["stress"][0], S, atol=1e-9)
    np.testing.assert_allclose(r["local_var"], V, atol=1e-12)


def test_batch_equals_alone(c1):
    """Each structure's result is the same alone and in a batch (bitwise:
    no float atomics, fixed reduction orders)."""
    ogp, b2a, ggp, calc = c1
    items = [syn.fcc_al(seed=s) for s in (1100, 1101, 1102)]
    items.append(syn.fcc_al(n_cells=3, seed=1103))
    batch = gpu_predict(ggp, calc, items)
    off = batch["offsets"]
    for k, it in enumerate(items):
        alone = gpu_predict(ggp, calc, [it])
        assert alone["energy"][0] == batch["energy"][k]
        np.testing.assert_array_equal(alone["forces"],
                                      batch["forces"][off[k]:off[k + 1]])
        np.testing.assert_array_equal(alone["stress"][0], batch["stress"][k])
        np.testing.assert_array_equal(alone["local_var"],
                                      batch["local_var"][off[k]:off[k + 1]])


def test_deterministic_repeat(c1):
    ogp, b2a, ggp, calc = c1
    it = [syn.fcc_al(seed=1105)]
    a = gpu_predict(ggp, calc, it)
    b = gpu_predict(ggp, calc, it)
    for k in ("energy", "forces", "stress", "local_var"):
        np.testing.assert_array_equal(a[k], b[k])


def test_forces_are_energy_gradient(c1):
    """Adjoint forces against central differences of the GPU energy."""
    ogp, b2a, ggp, calc = c1
    cell, sp, pos = syn.fcc_al(n_cells=2, seed=1107)
    r = gpu_predict(ggp, calc, [(cell, sp, pos)])
    h = 1e-4
    for atom, c in [(0, 0), (3, 2), (17, 1)]:
        p1 = pos.copy(); p1[atom, c] += h
        p2 = pos.copy(); p2[atom, c] -= h
        e1 = gpu_predict(ggp, calc, [(cell, sp, p1)])["energy"][0]
        e2 = gpu_predict(ggp, calc, [(cell, sp, p2)])["energy"][0]
        # tolerance of the reference's finite-difference tests
        # (test_kernels.cpp: delta 1e-4, tolerance 1e-4)
        assert abs(r["forces"][atom, c] + (e1 - e2) / (2 * h)) < 1e-4


def test_stale_model_raises():
    import flare_gb300 as fg
    calc = fg.B2(*b2_args(1, 4, 2, 5.0)[:5])
    gp = fg.SparseGP([fg.NormalizedDotProduct(1.0, 2)], 0.1, 0.1, 0.1)
    cell, sp, pos = syn.fcc_al(n_cells=2, seed=1)
    with pytest.raises(RuntimeError, match="L_inv must be up to date"):
        gp.predict_mean(fg.Structure(cell, sp, pos, 5.0, [calc]))


def test_species_out_of_range_raises(c1):
    ogp, b2a, ggp, calc = c1
    import flare_gb300 as fg
    cell, sp, pos = syn.fcc_al(n_cells=2, seed=1)
    sp = sp.copy()
    sp[3] = 4
    with pytest.raises(ValueError):
        ggp.predict_batch([fg.Structure(cell, sp, pos, 5.0, [calc])])


def test_autograd_energy_gradient_is_minus_forces(c1):
    import torch
    import flare_gb300 as fg
    from flare_gb300.autograd import energy
    ogp, b2a, ggp, calc = c1
    items = [syn.fcc_al(seed=1110), syn.fcc_al(seed=1111)]
    strucs = [fg.Structure(c, s, p, 5.0, [calc]) for c, s, p in items]
    pos = torch.from_numpy(np.concatenate([p for _, _, p in items])).cuda()
    pos.requires_grad_(True)
    e = energy(pos, ggp, strucs)
    w = torch.tensor([1.0, -2.5], dtype=torch.float64, device="cuda")
    (g,) = torch.autograd.grad((e * w).sum(), pos)
    r = ggp.predict_batch(strucs)
    F = r["forces"]
    np.testing.assert_allclose(g[:256].cpu().numpy(), -F[:256] * 1.0, atol=1e-12)
    np.testing.assert_allclose(g[256:].cpu().numpy(), -F[256:] * -2.5, atol=1e-12)
    np.testing.assert_allclose(e.detach().cpu().numpy(), r["energy"], rtol=0,
                               atol=0)


@pytest.mark.parametrize("slices", [None, (9, 9), (8, 8), (7, 6)])
@pytest.mark.parametrize("power", [2, 1])
def test_mixed_precision_within_budget(power, slices):
    """Mixed path against the FP64 path on an FCC model (|alpha| ~ 1e4):
    energy and local variance come from the tensor-core GEMMs with exact
    integer slicing, forces from the alpha-folded FP32 GEMM and the FP32
    adjoint.  At every slice count the model may run (the probes' choice
    when `slices` is None; forced otherwise) the stated budget holds:
    energy <= 1e-6 eV/atom, local variance <= 1e-8 sigma^2, force MAE <=
    1e-4 eV/A, stress 1e-5 eV/A^3; at 9 slices (54 bits) energy and
    variance are FP64-level (1e-8 eV/atom, 1e-11)."""
    ogp, b2a = c1_model(n_train=8, n_sparse=120, power=power)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    if slices:
        ggp.set_slices(*slices)
    plan = ggp.mixed_plan()
    sig2 = ogp.kernels[0].sigma ** 2
    if slices:
        assert (plan["kernel_slices"], plan["variance_slices"]) == slices
    else:
        assert plan["kernel_slices"] in (7, 8, 9), plan
        assert plan["variance_slices"] in (6, 7, 8, 9), plan
        assert plan["slice_err_ev_per_atom"] <= 1e-7, plan
        assert plan["variance_slice_err"] <= 5e-9 * sig2, plan
    items = [syn.fcc_al(seed=1120 + k) for k in range(3)]
    a = gpu_predict(ggp, calc, items, precision="fp64")
    b = gpu_predict(ggp, calc, items, precision="mixed")
    e_tol, v_tol = (1e-8, 1e-11) if slices == (9, 9) else (1e-6, 1e-8 * sig2)
    assert np.max(np.abs(a["energy"] - b["energy"])) / 256 <= e_tol
    np.testing.assert_allclose(b["local_var"], a["local_var"], rtol=0,
                               atol=v_tol)
    mae = np.abs(a["forces"] - b["forces"]).mean()
    assert mae <= 1e-4, mae
    np.testing.assert_allclose(b["stress"], a["stress"], atol=1e-5)


@pytest.mark.parametrize("power", [2, 1])
def test_mixed_guard_large_fold(power):
    """Ill-conditioned model (|alpha| ~ 1e9 from near-duplicate sparse
    environments; largest folded coefficient sigma^2 |sum alpha s^ s^T|
    ~ 1e5-1e6): the FP32-level force stage would err by ~0.1 eV/A, so the
    fold guard must switch the force product, mapped gradient and adjoint
    to FP64 level; forces then agree with the FP64 path to 1e-6 eV/A MAE
    and the oracle's energy to 1e-6 eV/atom."""
    from flare_gb300 import mapped
    ogp, b2a = small_two_species(seed=5, n_train=2, power=power)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    fmax, f64 = mapped.fold_guard(ggp)
    assert f64 and fmax > 200.0, (fmax, f64)
    cell, sp, pos = random_atoms(seed=55)
    E, F, Sg, V = oracle_predict(ogp, b2a, cell, sp, pos)
    b = gpu_predict(ggp, calc, [(cell, sp, pos)], precision="mixed")
    assert abs(b["energy"][0] - E) / len(sp) <= 1e-6
    assert np.abs(b["forces"] - F).mean() <= 1e-6
    np.testing.assert_allclose(b["local_var"], V, rtol=0, atol=1e-8)


def test_mixed_guard_keeps_fast_path():
    """A well-conditioned FCC model (largest folded coefficient ~6) stays on
    the FP32-level force stage."""
    from flare_gb300 import mapped
    ogp, b2a = c1_model(n_train=8, n_sparse=120)
    ggp, _ = to_gpu_sgp(ogp, b2a)
    fmax, f64 = mapped.fold_guard(ggp)
    assert not f64 and 0.0 < fmax < 200.0, (fmax, f64)


@pytest.mark.parametrize("power", [2, 1])
@pytest.mark.parametrize("multicut", [False, True])
def test_self_kernel_struc_matches_oracle(power, multicut):
    """NormalizedDotProduct::self_kernel_struc (normalized_dot_product.cpp:
    450-586) on a 16-atom, 2-species cell in a 4 A box (every atom its own
    neighbour through images) against the oracle's restatement of the
    reference loop; FP64, relative 1e-10 of the largest entry."""
    import flare_gb300 as fg
    S = 2
    cutoffs = (5.0 * np.ones((S, S)) + np.eye(S) - 1) if multicut else None
    b2a = b2_args(S, 3, 2, 5.0, cutoffs=cutoffs)
    cell, sp, pos = random_atoms(seed=17)
    st = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    ref = oracle.NormalizedDotProduct(1.3, power).self_kernel_struc(
        st.descriptors[0])
    calc = fg.B2(*b2a[:5], cutoffs=b2a[5])
    got = fg.NormalizedDotProduct(1.3, power).self_kernel_struc(
        fg.Structure(cell, sp, pos, 5.0, [calc]))
    np.testing.assert_allclose(got, ref, rtol=0,
                               atol=1e-10 * np.abs(ref).max())


def test_self_kernel_struc_fcc():
    """The same on a 108-atom FCC cell (3 x 3 x 3 cells, rc 4.5 A, one
    species), where neighbourhoods hold distinct atoms."""
    import flare_gb300 as fg
    b2a = b2_args(1, 6, 3, 4.5)
    cell, sp, pos = syn.fcc_al(n_cells=3, seed=11)
    st = oracle.Structure(cell, sp, pos, 4.5, [oracle.B2Settings(*b2a)])
    ref = oracle.NormalizedDotProduct(2.0, 2).self_kernel_struc(
        st.descriptors[0])
    calc = fg.B2(*b2a[:5], cutoffs=b2a[5])
    got = fg.NormalizedDotProduct(2.0, 2).self_kernel_struc(
        fg.Structure(cell, sp, pos, 4.5, [calc]))
    np.testing.assert_allclose(got, ref, rtol=0,
                               atol=1e-10 * np.abs(ref).max())


def test_predict_dtc_matches_oracle():
    """SparseGP::predict_DTC (sparse_gp.cpp:694-729): mean and the DTC
    variances of every output against the oracle (FP64; variances within
    1e-10 of the largest prior variance)."""
    import flare_gb300 as fg
    ogp, b2a = small_two_species(seed=5, n_train=2)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    ggp.R_inv = ogp.R_inv
    cell, sp, pos = random_atoms(seed=55)
    st = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    ogp.predict_DTC(st)
    g = fg.Structure(cell, sp, pos, 5.0, [calc])
    ggp.predict_DTC(g)
    np.testing.assert_allclose(g.mean_efs, st.mean_efs, rtol=0,
                               atol=1e-8 * np.abs(st.mean_efs).max())
    # the variance is K_self - Q_self + V_SOR with K_self and Q_self of
    # similar size (this model's L_inv is large): FP64 agreement is relative
    # to the terms, not to their difference
    ks = ogp.kernels[0].self_kernel_struc(st.descriptors[0])
    np.testing.assert_allclose(g.variance_efs, st.variance_efs, rtol=0,
                               atol=1e-10 * np.abs(ks).max())


@pytest.mark.parametrize("power", [2, 1])
@pytest.mark.parametrize("multicut", [False, True])
def test_struc_struc_matches_oracle(power, multicut):
    """NormalizedDotProduct::struc_struc (normalized_dot_product.cpp:216-448)
    between two 16-atom, 2-species cells against the oracle's restatement
    of the reference loop: every energy, force and stress entry, FP64,
    1e-10 of the largest entry."""
    import flare_gb300 as fg
    S = 2
    cutoffs = (5.0 * np.ones((S, S)) + np.eye(S) - 1) if multicut else None
    b2a = b2_args(S, 3, 2, 5.0, cutoffs=cutoffs)
    (c1, sp1, p1), (c2, sp2, p2) = random_atoms(seed=21), random_atoms(seed=22)
    sp2 = sp2[::-1].copy()
    ob2 = oracle.B2Settings(*b2a)
    o1 = oracle.Structure(c1, sp1, p1, 5.0, [ob2])
    o2 = oracle.Structure(c2, sp2, p2, 5.0, [ob2])
    ref = oracle.NormalizedDotProduct(1.3, power).struc_struc(
        o1.descriptors[0], o2.descriptors[0])
    calc = fg.B2(*b2a[:5], cutoffs=b2a[5])
    got = fg.NormalizedDotProduct(1.3, power).struc_struc(
        fg.Structure(c1, sp1, p1, 5.0, [calc]),
        fg.Structure(c2, sp2, p2, 5.0, [calc]))
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=0,
                               atol=1e-10 * np.abs(ref).max())


def test_struc_struc_fcc_different_sizes():
    """struc_struc between a 32-atom and a 108-atom FCC cell (rc 4.5 A, one
    species): rectangular blocks, distinct-atom neighbourhoods."""
    import flare_gb300 as fg
    b2a = b2_args(1, 5, 3, 4.5)
    c1, sp1, p1 = syn.fcc_al(n_cells=2, seed=31)
    c2, sp2, p2 = syn.fcc_al(n_cells=3, seed=32)
    ob2 = oracle.B2Settings(*b2a)
    ref = oracle.NormalizedDotProduct(2.0, 2).struc_struc(
        oracle.Structure(c1, sp1, p1, 4.5, [ob2]).descriptors[0],
        oracle.Structure(c2, sp2, p2, 4.5, [ob2]).descriptors[0])
    calc = fg.B2(*b2a[:5], cutoffs=b2a[5])
    got = fg.NormalizedDotProduct(2.0, 2).struc_struc(
        fg.Structure(c1, sp1, p1, 4.5, [calc]),
        fg.Structure(c2, sp2, p2, 4.5, [calc]))
    np.testing.assert_allclose(got, ref, rtol=0,
                               atol=1e-10 * np.abs(ref).max())


BASES = [("chebyshev", [0.5, 5.0]), ("weighted_chebyshev", [0.5, 5.0, 3.0]),
         ("equispaced_gaussians", [0.6, 5.0, 0.8]),
         ("weighted_positive_chebyshev", [0.5, 5.0, 3.0]),
         ("positive_chebyshev", [0.5, 5.0]), ("bessel", [0.0, 5.0]),
         ("fourier_quarter", [0.5, 5.0]), ("fourier_half", [0.5, 5.0]),
         ("fourier", [0.5, 5.0, 0.75])]


@pytest.mark.parametrize("basis,rh", BASES, ids=[b for b, _ in BASES])
def test_radial_bases_predict_matches_oracle(basis, rh):
    """Every radial basis of radial.cpp:6-336 through the whole path: a
    2-species model (per-pair cutoffs 4.5 / 5.0, so radial_hyps[1] is
    overwritten per pair as in b2.cpp:352) trained by the oracle, then B2,
    energy, forces, stress and local variance in FP64 against the oracle,
    and the mixed path within its budget."""
    import flare_gb300 as fg
    from helpers import lj_labels, oracle_model
    S = 2
    cut = np.array([[5.0, 4.5], [4.5, 5.0]])
    b2a = (basis, "quadratic", rh, [], [S, 4, 2], cut)
    strucs, labels, sparse = [], [], []
    for t in range(2):
        c, s_, p_ = random_atoms(seed=600 + t)
        strucs.append((c, s_, p_))
        labels.append(lj_labels(c, s_, p_, S))
        sparse.append([0, 3, 5, 8, 12])
    ogp, _ = oracle_model(strucs, labels, sparse, b2a, sigma=1.4, power=2,
                          noise=(0.3, 0.2, 0.4))
    ggp, calc = to_gpu_sgp(ogp, b2a)
    cell, sp, pos = random_atoms(seed=650)
    o = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    g = fg.Structure(cell, sp, pos, 5.0, [calc])
    B, _ = g.b2_values()
    ob = o.descriptors[0].atom_B2
    np.testing.assert_allclose(B.cpu().numpy(), ob, rtol=1e-11,
                               atol=1e-12 * np.abs(ob).max())
    E, F, Sg, V = oracle_predict(ogp, b2a, cell, sp, pos)
    a = gpu_predict(ggp, calc, [(cell, sp, pos)])
    assert abs(a["energy"][0] - E) <= 1e-9 * max(1, abs(E))
    Fs = max(1.0, np.abs(F).max())
    np.testing.assert_allclose(a["forces"], F, rtol=0, atol=1e-8 * Fs)
    np.testing.assert_allclose(a["stress"][0], Sg, rtol=0,
                               atol=1e-9 * max(1.0, np.abs(Sg).max()))
    np.testing.assert_allclose(a["local_var"], V, rtol=0, atol=1e-9)
    # mixed: this tiny-cell model is far from physical (|E| ~ 1e9 eV, forces
    # ~1e5 eV/A), so both bounds also carry a term relative to the values,
    # as the FP64 bounds above do
    b = gpu_predict(ggp, calc, [(cell, sp, pos)], precision="mixed")
    assert abs(b["energy"][0] - E) <= 1e-6 * len(sp) + 1e-11 * abs(E)
    assert np.abs(b["forces"] - F).mean() <= 1e-4 + 1e-9 * Fs


def test_structure_kernels_with_isolated_atom():
    """self_kernel_struc, struc_struc and predict_DTC when one atom has no
    neighbours (descriptor norm below 1e-8: its rows are skipped, as in the
    reference's empty-environment tests) against the oracle."""
    import flare_gb300 as fg
    ogp, b2a = small_two_species(seed=5, n_train=2)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    ggp.R_inv = ogp.R_inv
    rng_ = np.random.Generator(np.random.PCG64(91))
    cell = np.eye(3) * 20.0
    pos = np.vstack([rng_.uniform(0, 4.0, size=(9, 3)) + 2.0, [[14, 14, 14]]])
    sp = np.array([0, 1] * 5)
    ob2 = oracle.B2Settings(*b2a)
    o = oracle.Structure(cell, sp, pos, 5.0, [ob2])
    assert o.descriptors[0].atom_norms.min() < 1e-8
    k = fg.NormalizedDotProduct(ogp.kernels[0].sigma, 2)
    g = fg.Structure(cell, sp, pos, 5.0, [calc])
    ref = ogp.kernels[0].self_kernel_struc(o.descriptors[0])
    np.testing.assert_allclose(k.self_kernel_struc(g), ref, rtol=0,
                               atol=1e-10 * np.abs(ref).max())
    c2, s2, p2 = random_atoms(seed=92)
    o2 = oracle.Structure(c2, s2, p2, 5.0, [ob2])
    ref2 = ogp.kernels[0].struc_struc(o.descriptors[0], o2.descriptors[0])
    got2 = k.struc_struc(g, fg.Structure(c2, s2, p2, 5.0, [calc]))
    np.testing.assert_allclose(got2, ref2, rtol=0,
                               atol=1e-10 * np.abs(ref2).max())
    ogp.predict_DTC(o)
    ggp.predict_DTC(g)
    np.testing.assert_allclose(g.variance_efs, o.variance_efs, rtol=0,
                               atol=1e-10 * np.abs(ref).max())
