"""GPU: fgb_predict_host, the end-to-end entry (host buffers in and out).
It counts and range-checks the species on the host and copies the results
back before its one synchronisation; its results must be the bits of
fgb_predict on device buffers, and a species outside the model's range
must be refused as the device entry refuses it (the reference's
Structure/B2 reject such species: structure.cpp, b2.cpp)."""
import numpy as np
import pytest

from helpers import random_atoms, small_two_species, to_gpu_sgp
from flare_gb300.core import pack_structures

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model():
    import flare_gb300 as fg
    ogp, b2a = small_two_species(seed=8)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    structs = [fg.Structure(*random_atoms(seed=80 + k), 5.0, [calc])
               for k in range(3)]
    return ggp, calc, structs


def _device(m, packed, prec, species=None):
    import torch
    from flare_gb300 import _lib
    offsets, cells, pos, sp = packed
    if species is not None:
        sp = species
    S, N = len(offsets) - 1, int(offsets[-1])
    d = {k: torch.zeros(n, dtype=torch.float64, device="cuda")
         for k, n in (("e", S), ("f", 3 * N), ("s", 6 * S), ("v", N))}
    d_pos = torch.from_numpy(pos).cuda()
    d_sp = torch.from_numpy(sp).cuda()
    rc = _lib.lib().fgb_predict(m.h, S, _lib.ptr(offsets), _lib.ptr(cells),
                                _lib.ptr(d_pos), _lib.ptr(d_sp), 5.0, 0xF,
                                prec, _lib.ptr(d["e"]), _lib.ptr(d["f"]),
                                _lib.ptr(d["s"]), _lib.ptr(d["v"]),
                                _lib.stream_ptr())
    torch.cuda.synchronize()
    return rc, {k: v.cpu().numpy() for k, v in d.items()}


def _host(m, packed, prec, species=None):
    from flare_gb300 import _lib
    offsets, cells, pos, sp = packed
    if species is not None:
        sp = species
    S, N = len(offsets) - 1, int(offsets[-1])
    h = {k: np.full(n, np.nan) for k, n in (("e", S), ("f", 3 * N),
                                             ("s", 6 * S), ("v", N))}
    rc = _lib.lib().fgb_predict_host(m.h, S, _lib.ptr(offsets),
                                     _lib.ptr(cells), _lib.ptr(pos),
                                     _lib.ptr(sp), 5.0, 0xF, prec,
                                     _lib.ptr(h["e"]), _lib.ptr(h["f"]),
                                     _lib.ptr(h["s"]), _lib.ptr(h["v"]),
                                     _lib.stream_ptr())
    return rc, h


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_host_entry_gives_device_bits(model, precision):
    from flare_gb300 import _lib
    ggp, calc, structs = model
    m = ggp._device_model([calc])
    prec = {"fp64": _lib.FGB_PREC_FP64, "mixed": _lib.FGB_PREC_MIXED}[precision]
    packed = pack_structures(structs)
    rd, dev = _device(m, packed, prec)
    rh, host = _host(m, packed, prec)
    assert rd == 0 and rh == 0
    for k in dev:
        np.testing.assert_array_equal(host[k], dev[k])


def test_species_out_of_range_refused_by_both_entries(model):
    from flare_gb300 import _lib
    ggp, calc, structs = model
    m = ggp._device_model([calc])
    packed = pack_structures(structs)
    bad = packed[3].copy()
    bad[5] = 2          # the model has species 0 and 1
    for call in (_device, _host):
        rc, _ = call(m, packed, _lib.FGB_PREC_MIXED, species=bad)
        assert rc == _lib.FGB_EINVAL
        assert "species must lie in [0, 2)" in \
            _lib.lib().fgb_last_error().decode()
    # the model still predicts afterwards
    rc, _ = _host(m, packed, _lib.FGB_PREC_MIXED)
    assert rc == 0
