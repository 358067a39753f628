"""GPU: the no-allocation neighbour-list entry point.

fgb_nlist_build_noalloc serves callers that cannot allocate device memory
(a host program that keeps its own fixed device-memory budget, or a loop
that must not allocate between steps): it keeps its working memory in a
fixed array inside the library and writes into buffers the caller owns.
Its output must equal the allocating entry point's (fgb_nlist_build +
fgb_nlist_export) exactly — the same tolerance as the other neighbour-list
tests — on consecutive calls, which share that array.
"""
import ctypes

import numpy as np
import pytest

from helpers import random_atoms
from flare_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def noalloc(cell, pos, cutoff, max_pairs):
    import torch
    from flare_gb300 import _lib
    L = _lib.lib()
    n = len(pos)
    d_pos = torch.from_numpy(np.ascontiguousarray(pos, np.float64)).cuda()
    cnt = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    sidx = torch.full((max(max_pairs, 1),), -1, dtype=torch.int32, device="cuda")
    sh = torch.zeros((max(3 * max_pairs, 1),), dtype=torch.int32, device="cuda")
    rel = torch.zeros((max(4 * max_pairs, 1),), dtype=torch.float64, device="cuda")
    P = ctypes.c_longlong(-1)
    h_cell = np.ascontiguousarray(cell, np.float64).reshape(-1)
    rc = L.fgb_nlist_build_noalloc(_lib.ptr(h_cell), _lib.ptr(d_pos), n,
                                   float(cutoff), max_pairs, _lib.ptr(cnt),
                                   _lib.ptr(sidx), _lib.ptr(sh), _lib.ptr(rel),
                                   ctypes.byref(P), _lib.stream_ptr())
    torch.cuda.synchronize()
    _lib.check(rc, "fgb_nlist_build_noalloc")
    P = P.value
    return {"neighbor_count": cnt.cpu().numpy()[:n],
            "structure_indices": sidx.cpu().numpy()[:P],
            "shifts": sh.cpu().numpy()[:3 * P].reshape(P, 3),
            "relative_positions": rel.cpu().numpy()[:4 * P].reshape(P, 4)}


def allocating(cell, sp, pos, cutoff):
    import flare_gb300 as fg
    return fg.Structure(cell, sp, pos, cutoff, []).neighbor_arrays()


def test_noalloc_matches_allocating_path_on_consecutive_calls():
    cases = [syn.random_alloy(1000, seed=2100) + (5.5,),
             syn.fcc_al(seed=1100) + (5.0,),
             random_atoms(seed=11) + (5.0,)]
    for cell, sp, pos, rc in cases:
        got = noalloc(cell, pos, rc, max_pairs=200000)
        ref = allocating(cell, sp, pos, rc)
        for k in ("neighbor_count", "structure_indices", "shifts",
                  "relative_positions"):
            np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


def test_noalloc_rejects_oversize_inputs():
    cell = np.eye(3) * 100.0
    pos = np.zeros((8193, 3))
    with pytest.raises(ValueError, match="no-allocation limit"):
        noalloc(cell, pos, 5.0, max_pairs=10)


def test_noalloc_reports_needed_capacity():
    cell, sp, pos = syn.fcc_al(n_cells=2, seed=3)
    with pytest.raises(ValueError, match="output capacity"):
        noalloc(cell, pos, 5.0, max_pairs=10)
    # the next call with room succeeds and matches
    got = noalloc(cell, pos, 5.0, max_pairs=20000)
    ref = allocating(cell, sp, pos, 5.0)
    np.testing.assert_array_equal(got["relative_positions"],
                                  ref["relative_positions"])
