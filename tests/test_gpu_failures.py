"""GPU: the bounded waits of the tensor-core GEMMs end and report instead
of hanging.  A barrier that nothing arrives at times out within its poll
limit, the CTA's other waiter leaves through the abort flag, the call
returns FGB_ETIMEOUT, and the context stays usable: a mixed prediction
after it is bitwise the one before.  No fault, trap or hang is involved."""
import ctypes

import numpy as np
import pytest

from helpers import c1_model, to_gpu_sgp
from flare_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_context_survives():
    import flare_gb300 as fg
    from flare_gb300 import _lib
    ogp, b2a = c1_model(n_train=4, n_sparse=60)
    gp, calc = to_gpu_sgp(ogp, b2a)
    cell, sp, pos = syn.fcc_al(seed=1170)

    def predict():
        return gp.predict_batch([fg.Structure(cell, sp, pos, 5.0, [calc])],
                                precision="mixed")

    r0 = predict()
    how = (ctypes.c_int * 2)()
    rc = _lib.lib().fgb_wait_expiry_check(1 << 12, how, _lib.stream_ptr())
    assert rc == _lib.FGB_ETIMEOUT
    assert b"ran out" in _lib.lib().fgb_last_error()
    assert list(how) == [2, 1]     # timed out; left through the abort flag
    with pytest.raises(ValueError):
        _lib.check(_lib.lib().fgb_wait_expiry_check(0, None,
                                                    _lib.stream_ptr()))
    r1 = predict()
    for k in ("energy", "forces", "stress", "local_var"):
        np.testing.assert_array_equal(r1[k], r0[k])
