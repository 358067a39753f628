"""CPU: the mapped-model file layout — the coefficient rows' line breaks
(the mapping writer keeps its column count across species rows, the varmap
writer resets it: sparse_gp.cpp:1236-1259 vs :1309-1331) and the readers'
round trip through the oracle's restatement of the writer."""
import numpy as np

import oracle


def test_padded_rows_line_breaks():
    from flare_gb300.mapped import _padded_rows
    rows = [[1.0, -2.0, 3.0], [4.0, 0.0]]
    f = "%.16e"
    keep = _padded_rows(rows, reset_count=False)
    assert keep == ("  " + f % 1.0 + " " + f % -2.0 + "  " + f % 3.0 + "\n" +
                    "  " + f % 4.0 + " " + f % 0.0 + "\n")
    reset = _padded_rows(rows, reset_count=True)
    assert reset == ("  " + f % 1.0 + " " + f % -2.0 + "  " + f % 3.0 + "\n" +
                     "  " + f % 4.0 + " " + f % 0.0)
    # six values on one row: a break after the fifth
    six = _padded_rows([[1.0] * 6], reset_count=True)
    assert six.count("\n") == 1 and six.index("\n") == 5 * 24


def test_mapping_file_round_trip(tmp_path):
    from flare_gb300.mapped import read_mapping_file
    # 2 species, n_max 1, l_max 1: 3 radial pairs x 2 l = 6 descriptors
    S, N, L = 2, 1, 1
    nr = S * N
    nd = nr * (nr + 1) // 2 * (L + 1)          # 6
    size = nd * (nd + 1) // 2                  # 21
    r = np.random.default_rng(5)
    beta = np.zeros((S, nd, nd))
    for s in range(S):
        a = r.normal(size=(nd, nd))
        beta[s] = a + a.T
    iu = np.triu_indices(nd)
    fac = np.where(iu[0] == iu[1], 1.0, 2.0)
    coeffs = np.stack([beta[s][iu] * fac for s in range(S)])
    assert coeffs.shape == (S, size)
    text = oracle.write_mapping_text(coeffs, 2, [S, N, L], "chebyshev",
                                     "quadratic", [[5.0, 4.5], [4.5, 5.0]],
                                     "tester", "Thu Jan  1 00:00:00 2026")
    f = tmp_path / "lmp.flare"
    f.write_text(text)
    info = read_mapping_file(str(f))
    assert info["power"] == 2 and info["descriptor_settings"] == [S, N, L]
    np.testing.assert_array_equal(info["cutoffs"], [[5.0, 4.5], [4.5, 5.0]])
    # the file keeps 17 significant digits: the matrices come back exactly
    # up to the halving of the doubled off-diagonal entries
    np.testing.assert_allclose(info["beta"], beta, rtol=1e-15, atol=0)
