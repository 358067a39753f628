"""GPU: cell-list neighbour list bit-exact against the oracle's brute-force
list (structure.cpp:52-118), and B2 against the oracle (b2.cpp)."""
import numpy as np
import pytest

import oracle
from helpers import b2_args, random_atoms
from flare_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def cases():
    out = []
    out.append(("fcc256", *syn.fcc_al(seed=1100), 5.0))
    out.append(("alloy1000", *syn.random_alloy(1000, seed=2100), 5.5))
    out.append(("tiny_box_sweep3", *random_atoms(seed=11), 5.0))
    # skewed triclinic cell (reference sweep can be conservative here)
    c, s, p = syn.random_alloy(200, seed=7)
    sk = np.array([[1.0, 0.0, 0.0], [0.35, 1.0, 0.0], [0.2, -0.3, 1.0]])
    out.append(("triclinic", c @ sk, s, p @ sk, 5.0))
    # atoms outside the cell (wrapping) and one exactly on a face
    c, s, p = syn.fcc_al(n_cells=3, seed=5)
    p = p + np.array([16.2, -8.1, 3 * 4.05 * 2])
    p[0] = [0.0, 0.0, 0.0]
    out.append(("unwrapped", c, s, p, 5.0))
    out.append(("sparse_gas", np.eye(3) * 30.0, np.zeros(3, int),
                np.array([[0, 0, 0], [1, 1, 1], [15, 15, 15.]]), 5.0))
    # fractional coordinates that wrap to exactly 1.0 (a tiny negative
    # coordinate): the atom's raw bin is the top one, in a cell whose bins
    # are staged per bin and in a tiny cell searched atom by atom
    for name, (c, s, p) in (("face_rounding", syn.random_alloy(300, seed=9)),
                            ("face_rounding_tiny", random_atoms(seed=12))):
        p = p.copy()
        p[0] = [-1e-18, 0.5 * c[1, 1], -1e-17]
        p[1] = [0.25 * c[0, 0], -3e-18, 0.5 * c[2, 2]]
        out.append((name, c, s, p, 5.0))
    out.append(("cluster_in_vacuum", *dense_cluster(), 5.0))
    return out


def dense_cluster(seed=13):
    """120 atoms at 0.2 atoms/A^3 in the middle of a 40 A cell: about 100
    neighbours per atom where the cell's mean density suggests one, so a
    single-pass build overflows its per-atom slots and the list is built
    again with a count pass."""
    c, s, p = syn.random_alloy(120, density=0.2, dmin=1.2, seed=seed)
    return np.eye(3) * 40.0, s, p + 16.0


@pytest.mark.parametrize("case", cases(), ids=lambda c: c[0])
def test_neighbor_list_bit_exact(case):
    import flare_gb300 as fg
    name, cell, sp, pos, rc = case
    o = oracle.Structure(cell, sp, pos, rc, [])
    g = fg.Structure(cell, sp, pos, rc, [])
    a = g.neighbor_arrays()
    np.testing.assert_array_equal(a["neighbor_count"], o.neighbor_count)
    np.testing.assert_array_equal(a["structure_indices"], o.structure_indices)
    np.testing.assert_array_equal(a["shifts"], o.shifts)
    # bit-exact relative vectors and distances
    np.testing.assert_array_equal(a["relative_positions"], o.relative_positions)
    np.testing.assert_array_equal(a["wrapped_positions"], o.wrapped_positions)


def test_empty_structure_and_isolated_atom():
    import flare_gb300 as fg
    g = fg.Structure(np.eye(3) * 30.0, [0], [[1.0, 2.0, 3.0]], 5.0, [])
    a = g.neighbor_arrays()
    assert a["neighbor_count"].tolist() == [0]


def test_nonfinite_positions_raise():
    import flare_gb300 as fg
    g = fg.Structure(np.eye(3) * 10.0, [0, 0], [[0, 0, 0], [np.nan, 1, 1]],
                     5.0, [])
    with pytest.raises(ValueError):
        g.neighbor_arrays()


@pytest.mark.parametrize("S,nmax,lmax,cut", [(1, 8, 3, "quadratic"),
                                             (2, 8, 4, "quadratic"),
                                             (2, 3, 2, "cosine"),
                                             (1, 10, 6, "quadratic"),
                                             (3, 4, 10, "polynomial")])
def test_b2_matches_oracle(S, nmax, lmax, cut):
    import flare_gb300 as fg
    cell, sp, pos = syn.random_alloy(150, fractions=[1.0 / S] * S, seed=31 + S)
    ch = [6.0] if cut == "polynomial" else []
    args = ("chebyshev", cut, [0.0, 5.0], ch, [S, nmax, lmax])
    o = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*args)],
                         compute_dervs=False)
    g = fg.Structure(cell, sp, pos, 5.0, [fg.B2(*args)])
    B, n = g.b2_values()
    ob = o.descriptors[0].atom_B2
    np.testing.assert_allclose(B.cpu().numpy(), ob, rtol=1e-11,
                               atol=1e-12 * np.abs(ob).max())
    np.testing.assert_allclose(n.cpu().numpy(), o.descriptors[0].atom_norms,
                               rtol=1e-12)


def test_b2_per_pair_cutoff_matrix():
    """b2.cpp:274-277: pairs beyond cutoffs(s_i, s_j) are skipped."""
    import flare_gb300 as fg
    cell, sp, pos = random_atoms(seed=21)
    cut = 5.0 * np.ones((2, 2)) + np.eye(2) - 1
    args = b2_args(2, 3, 2, 5.0, cutoffs=cut)
    o = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*args)],
                         compute_dervs=False)
    g = fg.Structure(cell, sp, pos, 5.0, [fg.B2(*args[:5], cutoffs=cut)])
    B, _ = g.b2_values()
    np.testing.assert_allclose(B.cpu().numpy(), o.descriptors[0].atom_B2,
                               rtol=1e-11, atol=1e-13)


def test_b2_stored_gradients_match_oracle():
    """fgb_b2_forward_dervs, the reference's stored forward-mode gradients
    (compute_b2, b2.cpp:181-242): dB2/dr per neighbour pair and component
    and force_dots = dB2/dr . B2, against the oracle's
    descriptor_force_dervs / descriptor_force_dots (one species, so the
    oracle's species blocks are in atom order)."""
    import torch
    import flare_gb300 as fg
    from flare_gb300._lib import check, lib, ptr, stream_ptr
    b2a = b2_args(1, 6, 3, 4.5)
    cell, sp, pos = syn.fcc_al(n_cells=2, seed=5)
    o = oracle.Structure(cell, sp, pos, 4.5, [oracle.B2Settings(*b2a)])
    calc = fg.B2(*b2a[:5], cutoffs=b2a[5])
    g = fg.Structure(cell, sp, pos, 4.5, [calc])
    N, nd, P = len(sp), calc.n_descriptors, g.n_neighbors
    dev = "cuda"
    B2 = torch.zeros((N, nd), dtype=torch.float64, device=dev)
    nrm = torch.zeros(N, dtype=torch.float64, device=dev)
    dB2 = torch.zeros((3 * P, nd), dtype=torch.float64, device=dev)
    fdot = torch.zeros(3 * P, dtype=torch.float64, device=dev)
    d = g._inputs()
    check(lib().fgb_b2_forward_dervs(calc.handle, g.nlist().h,
                                     ptr(d["species"]), ptr(B2), ptr(nrm),
                                     ptr(dB2), ptr(fdot), stream_ptr()),
          "b2_forward_dervs")
    ov = o.descriptors[0]
    ref = ov.descriptor_force_dervs[0]
    assert ref.shape == (3 * P, nd)
    np.testing.assert_allclose(dB2.cpu().numpy(), ref, rtol=0,
                               atol=1e-11 * np.abs(ref).max())
    np.testing.assert_allclose(fdot.cpu().numpy(), ov.descriptor_force_dots[0],
                               rtol=0, atol=1e-11 * np.abs(
                                   ov.descriptor_force_dots[0]).max())
    np.testing.assert_allclose(B2.cpu().numpy(), ov.atom_B2, rtol=1e-11,
                               atol=1e-12 * np.abs(ov.atom_B2).max())


def test_prediction_after_slot_overflow():
    """The prediction path builds its list without a count pass; on the
    dense cluster an atom overflows its slots, the call is repeated with a
    count pass, and energy, forces and stress match the oracle."""
    import flare_gb300 as fg
    from helpers import small_two_species, to_gpu_sgp
    ogp, b2a = small_two_species(seed=4)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    cell, sp, pos = dense_cluster()
    o = oracle.Structure(cell, sp, pos, 5.0, [oracle.B2Settings(*b2a)])
    ogp.predict_mean(o)
    m = o.mean_efs
    E, F, S = m[0], m[1:-6].reshape(-1, 3), m[-6:]
    for _ in range(2):   # the second call starts from the doubled slots
        r = ggp.predict_batch([fg.Structure(cell, sp, pos, 5.0, [calc])],
                              precision="fp64")
        assert abs(r["energy"][0] - E) <= 1e-9 * max(1.0, abs(E))
        np.testing.assert_allclose(r["forces"], F, rtol=0,
                                   atol=1e-8 * max(1.0, np.abs(F).max()))
        np.testing.assert_allclose(r["stress"][0], S, rtol=0,
                                   atol=1e-10 * max(1.0, np.abs(S).max()))
