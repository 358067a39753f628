"""GPU: the tile-shape autotuner of the sliced tensor-core GEMMs — every
candidate shape of the kernel, variance and force GEMMs gives the same
predictions bit for bit, the tuner times every candidate once per problem
shape and keeps the fastest, and later calls reuse the choice."""
import numpy as np
import pytest

from helpers import c1_model, to_gpu_sgp
from flare_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

KEYS = ("energy", "forces", "stress", "local_var")


@pytest.fixture(scope="module")
def setup():
    ogp, b2a = c1_model(n_train=8, n_sparse=120, power=2)
    gp, calc = to_gpu_sgp(ogp, b2a)
    items = [syn.fcc_al(seed=1500 + k) for k in range(4)]
    return gp, calc, items


def predict(gp, calc, items):
    import flare_gb300 as fg
    strucs = [fg.Structure(c, s, p, 5.0, [calc]) for c, s, p in items]
    return gp.predict_batch(strucs, precision="mixed")


def test_every_candidate_gives_identical_results(setup):
    from flare_gb300 import autotune as at
    gp, calc, items = setup
    at.set_mode(False)
    try:
        base = predict(gp, calc, items)
        for op, shapes in at.CANDIDATES.items():
            for c in range(len(shapes)):
                at.force(op, c)
                r = predict(gp, calc, items)
                for k in KEYS:
                    np.testing.assert_array_equal(r[k], base[k],
                                                  err_msg=f"{op} {c} {k}")
            at.force(op, None)
    finally:
        for op in at.OPS:
            at.force(op, None)
        at.set_mode(True)


def test_tuner_times_each_candidate_once_per_shape(setup):
    from flare_gb300 import autotune as at
    gp, calc, items = setup
    at.clear()
    at.set_mode(True)
    r1 = predict(gp, calc, items)
    table = at.table()
    assert {e["op"] for e in table} == set(at.OPS), table
    # the 64-row tiles exist for 8 slices and fewer only
    plan = gp.mixed_plan()
    n64 = {"kernel_gemm": 0 if plan["kernel_slices"] == 9 else 1,
           "variance_gemm": 0 if plan["variance_slices"] == 9 else 1}
    for e in table:
        expect = len(at.CANDIDATES[e["op"]])
        if e["op"] in n64:
            expect = 2 + n64[e["op"]]
        assert len(e["ms"]) == expect, e
        assert all(x > 0 for x in e["ms"]), e
        assert e["choice"] == int(np.argmin(e["ms"])), e
    r2 = predict(gp, calc, items)
    assert len(at.table()) == len(table)      # no new shapes, no re-timing
    for k in KEYS:
        np.testing.assert_array_equal(r1[k], r2[k], err_msg=k)
