"""GPU: parity at the alloy1000 workload — 2 species, B2 chebyshev/quadratic
[2, 8, 4] (n_d = 680), rc 5.5 A, NormalizedDotProduct sigma 2 power 2, about
1,000 sparse environments per species — the configuration the throughput
figures are quoted on, against the FP64 CPU oracle.

The oracle model is trained on two of the workload's training structures
(seeds 2000-2001) with the workload's sparse choice (seed 2200): prediction
shapes and cost (n_d, sparse environments per species) do not depend on the
training-set size.  The GPU path predicts with the oracle's weights, so every
difference below is the prediction path's own.  Reference functions:
SparseGP::predict_local_uncertainties (sparse_gp.cpp:731-757),
compute_cluster_uncertainties (sparse_gp.cpp:94-139), envs_struc
(normalized_dot_product.cpp:117-214), the B2 descriptor (b2.cpp:181-399) and
the calculator's post-processing (calculator.py:57-122).
"""
import numpy as np
import pytest

import oracle
from helpers import alloy_oracle_model, to_gpu_sgp
from flare_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

RC = wl.ALLOY["rc"]
SIG = wl.ALLOY["sigma"]

# FP64 path against the oracle.  sum_s |alpha_s k_is| reaches ~1e6 eV per
# atom on this model, so two FP64 evaluations in different summation orders
# differ by ~1e6 x 2^-53 x sqrt(M_s) ~ 1e-8 eV per atom at most.
E64_TOL = 1e-7     # eV per atom
F64_TOL = 1e-7     # eV/A, per component
S64_TOL = 1e-9     # eV/A^3
V64_TOL = 1e-11    # local variance
# Mixed path against the oracle: the stated budget (energy 1e-6 eV/atom,
# force MAE 1e-4 eV/A); local variance and the calculator's local std
# (sqrt|var| / sigma, the quantity compared with the 0.05 flag threshold).
EMIX_TOL = 1e-6    # eV per atom
FMIX_MAE = 1e-4    # eV/A
SMIX_TOL = 1e-5    # eV/A^3
VMIX_TOL = 4e-8    # local variance, 1e-8 of the prior variance sigma^2
STDMIX_TOL = 1e-6  # local std (dimensionless)


@pytest.fixture(scope="module")
def alloy():
    ogp, b2a = alloy_oracle_model()
    ggp, calc = to_gpu_sgp(ogp, b2a, cutoff=RC)
    tests = [wl.alloy_structure(wl.ALLOY["test_seed0"] + k) for k in range(2)]
    ref = []
    for cell, sp, pos in tests:
        st = oracle.Structure(cell, sp, pos, RC, [oracle.B2Settings(*b2a)])
        ogp.predict_local_uncertainties(st)
        m = st.mean_efs
        var = oracle.sort_variances(st, st.local_uncertainties[0])
        ref.append((m[0], m[1:-6].reshape(-1, 3), m[-6:], var))
    return ogp, b2a, ggp, calc, tests, ref


class Atoms:
    def __init__(self, cell, numbers, positions):
        self.cell = cell
        self.numbers = numbers
        self.positions = positions


def _predict(ggp, calc, tests, precision):
    import flare_gb300 as fg
    strucs = [fg.Structure(c, s, p, RC, [calc]) for c, s, p in tests]
    return ggp.predict_batch(strucs, precision=precision)


def _split(r, tests):
    out, a0 = [], 0
    for k, (_, sp, _) in enumerate(tests):
        n = len(sp)
        out.append((r["energy"][k], r["forces"][a0:a0 + n], r["stress"][k],
                    r["local_var"][a0:a0 + n]))
        a0 += n
    return out


def test_alloy_model_shape(alloy):
    ogp, b2a, ggp, calc, tests, ref = alloy
    assert ogp.sparse_descriptors[0].n_descriptors == 680
    counts = list(ogp.sparse_descriptors[0].n_clusters_by_type)
    assert len(counts) == 2 and min(counts) >= 950, counts
    assert all(len(sp) == 1000 for _, sp, _ in tests)


def test_alloy_fp64_matches_oracle(alloy):
    ogp, b2a, ggp, calc, tests, ref = alloy
    got = _split(_predict(ggp, calc, tests, "fp64"), tests)
    for (E, F, S, V), (e, f, s, v), (_, sp, _) in zip(ref, got, tests):
        n = len(sp)
        assert abs(e - E) / n <= E64_TOL, (e, E)
        np.testing.assert_allclose(f, F, rtol=0, atol=F64_TOL)
        np.testing.assert_allclose(s, S, rtol=0, atol=S64_TOL)
        np.testing.assert_allclose(v, V, rtol=0, atol=V64_TOL)


@pytest.mark.parametrize("slices", [None, (8, 8), (7, 6)])
def test_alloy_mixed_matches_oracle(alloy, slices):
    """The mixed path (double-float descriptor, exact-slicing tensor-core
    kernel and variance GEMMs, FP32-level force GEMM, FP32 adjoint)
    against the oracle itself, not against this library's FP64 path: at the
    slice counts the probes choose (None) and forced to 8/8 and to the
    fewest the path takes, 7 for the kernel GEMM and 6 for the variance."""
    ogp, b2a, ggp, calc, tests, ref = alloy
    ggp.set_slices(*(slices or (0, 0)))
    plan = ggp.mixed_plan()
    if slices:
        assert (plan["kernel_slices"], plan["variance_slices"]) == slices
    else:
        assert plan["kernel_slices"] in (7, 8, 9), plan
        assert plan["variance_slices"] in (6, 7, 8, 9), plan
    assert not plan["fp64_forces"], plan   # alloy folds stay below the guard
    got = _split(_predict(ggp, calc, tests, "mixed"), tests)
    for (E, F, S, V), (e, f, s, v), (_, sp, _) in zip(ref, got, tests):
        n = len(sp)
        assert abs(e - E) / n <= EMIX_TOL, (e, E)
        assert np.abs(f - F).mean() <= FMIX_MAE
        np.testing.assert_allclose(s, S, rtol=0, atol=SMIX_TOL)
        np.testing.assert_allclose(v, V, rtol=0, atol=VMIX_TOL)
        std = np.sqrt(np.abs(v)) / SIG
        STD = np.sqrt(np.abs(V)) / SIG
        assert np.abs(std - STD).max() <= STDMIX_TOL


def test_alloy_calculator_matches_oracle(alloy):
    """SGP_Calculator results (energy, forces, ASE-order stress, local stds)
    on the mixed path against the oracle's calculator post-processing."""
    import flare_gb300 as fg
    from flare_gb300.sparse_gp import SGP_Wrapper
    ogp, b2a, ggp, calc, tests, ref = alloy
    ggp.set_slices(0, 0)
    cell, sp, pos = tests[0]
    st = oracle.Structure(cell, sp, pos, RC, [oracle.B2Settings(*b2a)])
    ogp.predict_local_uncertainties(st)
    want = oracle.calculator_results(st, "local", SIG)
    k = ggp.kernels[0]
    w = SGP_Wrapper([k], [calc], RC, ggp.energy_noise, ggp.force_noise,
                    ggp.stress_noise, {13: 0, 29: 1}, variance_type="local")
    w.sparse_gp = ggp
    c = fg.SGP_Calculator(w)
    prev = fg.get_precision()
    fg.set_precision("mixed")
    try:
        c.calculate(Atoms(cell, np.where(np.asarray(sp) == 0, 13, 29), pos))
    finally:
        fg.set_precision(prev)
    got = c.results
    n = len(sp)
    assert abs(got["energy"] - want["energy"]) / n <= EMIX_TOL
    assert np.abs(got["forces"] - want["forces"]).mean() <= FMIX_MAE
    np.testing.assert_allclose(got["stress"], want["stress"], atol=SMIX_TOL)
    np.testing.assert_allclose(got["stds"], want["stds"], atol=STDMIX_TOL)
