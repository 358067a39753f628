"""GPU: SparseGP with two kernels (two B2 descriptors of different settings
and cutoffs, a power-2 and a power-1 NormalizedDotProduct) against the FP64
oracle.  The reference stacks the kernels' sparse sets: the mean is the sum
of each kernel's K_i^T alpha_i (sparse_gp.cpp:643-665), each kernel's local
variances use its own diagonal block of L_inv (sparse_gp.cpp:94-139), and the
SOR / DTC variances take the stacked kernel matrix with the full R_inv,
Kuu^-1 and Sigma (sparse_gp.cpp:667-729)."""
import numpy as np
import pytest

import oracle
from helpers import b2_args, lj_labels
from flare_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def alloy48(seed):
    """48-atom random 2-species cell at 0.06 atoms/A^3 (10.2 A box)."""
    return syn.random_alloy(48, density=0.06, fractions=(0.5, 0.5), dmin=1.8,
                            seed=seed)


B2A = b2_args(2, 3, 2, 5.0)
B2B = b2_args(2, 4, 1, 4.0, cutoff_function="cosine")
KERN = [(1.5, 2), (0.8, 1)]


@pytest.fixture(scope="module")
def two_kernels():
    import flare_gb300 as fg
    ob = [oracle.B2Settings(*B2A), oracle.B2Settings(*B2B)]
    ogp = oracle.SparseGP([oracle.NormalizedDotProduct(s, p) for s, p in KERN],
                          0.3, 0.2, 0.4)
    r = np.random.Generator(np.random.PCG64(71))
    for t in range(3):
        cell, sp, pos = alloy48(700 + t)
        E, F, St = lj_labels(cell, sp, pos, 2)
        st = oracle.Structure(cell, sp, pos, 5.0, ob)
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        st.stresses = St
        ogp.add_training_structure(st)
        ogp.add_specific_environments(
            st, sorted(r.choice(len(sp), size=8, replace=False).tolist()))
    ogp.update_matrices_QR()
    calcs = [fg.B2(*B2A[:5]), fg.B2(*B2B[:5])]
    ggp = fg.SparseGP([fg.NormalizedDotProduct(s, p) for s, p in KERN],
                      0.3, 0.2, 0.4)
    cds = []
    for osd in ogp.sparse_descriptors:
        cd = fg.ClusterDescriptor(osd.n_types, osd.n_descriptors)
        cd.descriptors = [np.asarray(d) for d in osd.descriptors]
        cd.descriptor_norms = [np.asarray(d) for d in osd.descriptor_norms]
        cd.n_clusters_by_type = list(osd.n_clusters_by_type)
        cd.cumulative_type_count = list(osd.cumulative_type_count)
        cd.n_clusters = osd.n_clusters
        cds.append(cd)
    ggp.set_weights(cds, ogp.alpha, ogp.L_inv, calcs)
    ggp.R_inv = ogp.R_inv
    ggp.Sigma = ogp.Sigma
    ggp.Kuu_inverse = ogp.Kuu_inverse
    cell, sp, pos = alloy48(777)
    return ogp, ggp, calcs, (cell, sp, pos)


def _pair(two_kernels):
    import flare_gb300 as fg
    ogp, ggp, calcs, (cell, sp, pos) = two_kernels
    o = oracle.Structure(cell, sp, pos, 5.0,
                         [oracle.B2Settings(*B2A), oracle.B2Settings(*B2B)])
    g = fg.Structure(cell, sp, pos, 5.0, calcs)
    return ogp, ggp, o, g


def _close_efs(g, o, tol=1e-8):
    scale = max(1.0, np.abs(o).max())
    np.testing.assert_allclose(g, o, rtol=0, atol=tol * scale)


def test_two_kernel_mean_and_local_uncertainties(two_kernels):
    ogp, ggp, o, g = _pair(two_kernels)
    ogp.predict_local_uncertainties(o)
    ggp.predict_local_uncertainties(g)
    _close_efs(g.mean_efs, o.mean_efs)
    assert len(g.local_uncertainties) == 2
    for a, b in zip(g.local_uncertainties, o.local_uncertainties):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-10)
    ogp2, ggp2, o2, g2 = _pair(two_kernels)
    ggp2.predict_mean(g2)
    _close_efs(g2.mean_efs, o.mean_efs)


def test_two_kernel_sor(two_kernels):
    ogp, ggp, o, g = _pair(two_kernels)
    ogp.predict_SOR(o)
    ggp.predict_SOR(g)
    _close_efs(g.mean_efs, o.mean_efs)
    np.testing.assert_allclose(g.variance_efs, o.variance_efs, rtol=1e-8,
                               atol=1e-10)


def test_two_kernel_dtc(two_kernels):
    ogp, ggp, o, g = _pair(two_kernels)
    ogp.predict_DTC(o)
    ggp.predict_DTC(g)
    _close_efs(g.mean_efs, o.mean_efs)
    np.testing.assert_allclose(g.variance_efs, o.variance_efs, rtol=1e-7,
                               atol=1e-9)


def test_two_kernel_mixed_within_budget(two_kernels):
    """The mixed path per kernel, summed: energy within 1e-6 eV/atom and
    force MAE within 1e-4 eV/A of the oracle."""
    ogp, ggp, o, g = _pair(two_kernels)
    ogp.predict_mean(o)
    r = ggp.predict_batch([g], precision="mixed")
    n = g.noa
    assert abs(r["energy"][0] - o.mean_efs[0]) / n <= 1e-6
    F = o.mean_efs[1:-6].reshape(-1, 3)
    assert np.abs(r["forces"] - F).mean() <= 1e-4
