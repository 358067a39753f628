"""GPU: continuous batching — requests of uneven sizes and species mixes
arriving while others run are batched with memory admission, their work
overlaps on two workers, and every result equals the same structure
predicted alone (bitwise: no float atomics, fixed reduction orders)."""
import threading
import time

import numpy as np
import pytest

from helpers import small_two_species, to_gpu_sgp
from flare_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def requests(n, seed=4000):
    r = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n):
        N = int(np.exp(r.uniform(np.log(16), np.log(300))))
        S = int(r.integers(1, 3))
        fr = r.dirichlet(np.ones(S))
        fr = np.concatenate([fr, np.zeros(2 - S)])
        cell, sp, pos = syn.random_alloy(N, density=r.uniform(0.05, 0.09),
                                         fractions=fr, seed=4100 + k)
        out.append((cell, sp, pos))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_serving_same_alone_and_in_the_mix(precision):
    import flare_gb300 as fg
    from flare_gb300.serving import Server
    ogp, b2a = small_two_species(seed=21, n_train=3)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    reqs = requests(40)
    srv = Server(ggp, calc, 5.0, n_workers=2, memory_budget_gb=2.0,
                 max_structures=16, precision=precision)
    ids = [None] * len(reqs)

    def producer():
        # a burst of 16 (queued while the workers run their first batches),
        # then Poisson arrivals that land while other batches are on the GPU
        r = np.random.Generator(np.random.PCG64(7))
        for k, (cell, sp, pos) in enumerate(reqs):
            ids[k] = srv.submit(cell, sp, pos)
            if k >= 16:
                time.sleep(float(r.exponential(0.002)))

    t = threading.Thread(target=producer)
    t.start()
    t.join()
    got = [srv.result(i) for i in ids]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    assert st["batches"] < len(reqs)          # requests were batched
    for (cell, sp, pos), g in zip(reqs, got):
        alone = ggp.predict_batch([fg.Structure(cell, sp, pos, 5.0, [calc])],
                                  precision=precision)
        assert g["energy"] == alone["energy"][0]
        np.testing.assert_array_equal(g["forces"], alone["forces"])
        np.testing.assert_array_equal(g["stress"], alone["stress"][0])
        np.testing.assert_array_equal(g["local_var"], alone["local_var"])
    lat = np.array([g["latency_ms"] for g in got])
    assert np.all(lat > 0)


def test_admission_refuses_oversize_request():
    from flare_gb300.serving import Server
    ogp, b2a = small_two_species(seed=22, n_train=2)
    ggp, calc = to_gpu_sgp(ogp, b2a)
    srv = Server(ggp, calc, 5.0, n_workers=1, memory_budget_gb=0.001)
    cell, sp, pos = syn.random_alloy(2000, seed=1)
    with pytest.raises(ValueError, match="memory budget"):
        srv.submit(cell, sp, pos)
    srv.close()
