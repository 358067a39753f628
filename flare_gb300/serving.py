"""Continuous-batching prediction server (the library's native worker pool,
fgb_serve_* in include/flaregb.h) with a small Python front end."""
import ctypes
import time

import numpy as np

from . import _lib
from ._lib import check, lib, ptr
from .core import _prec, get_precision


class Server:
    """Server(sgp, calc, n_workers=2, memory_budget_gb=8, max_structures=64,
    want=E|F|S|local var, precision=None).

    ``submit(cell, species, positions)`` returns a request id;
    ``result(id)`` blocks until that request is done and returns a dict with
    energy, forces, stress (flare order), local_var and latency_ms.
    """

    def __init__(self, sgp, calc, cutoff, n_workers=2, memory_budget_gb=8.0,
                 max_structures=64, want=0xF, precision=None):
        m = sgp._device_model([calc])
        h = ctypes.c_void_p()
        check(lib().fgb_serve_start(ctypes.byref(h), m.h, int(n_workers),
                                    int(memory_budget_gb * 2 ** 30),
                                    int(max_structures), float(cutoff),
                                    int(want), _prec[precision or get_precision()]),
              "serve")
        self.h = h
        self._model = m
        self._n = {}

    def submit(self, cell, species, positions):
        cell = np.ascontiguousarray(cell, np.float64).reshape(9)
        pos = np.ascontiguousarray(positions, np.float64).reshape(-1, 3)
        sp = np.ascontiguousarray(species, np.int32).reshape(-1)
        rid = ctypes.c_longlong()
        check(lib().fgb_serve_submit(self.h, len(sp), ptr(cell), ptr(pos),
                                     ptr(sp), ctypes.byref(rid)), "submit")
        self._n[rid.value] = len(sp)
        return rid.value

    def poll(self, rid):
        n = self._n[rid]
        done = ctypes.c_int()
        e = np.zeros(1)
        f = np.zeros((max(n, 1), 3))
        s = np.zeros(6)
        v = np.zeros(max(n, 1))
        lat = ctypes.c_double()
        check(lib().fgb_serve_poll(self.h, rid, ctypes.byref(done), ptr(e),
                                   ptr(f), ptr(s), ptr(v), ctypes.byref(lat)),
              "poll")
        if not done.value:
            return None
        del self._n[rid]
        return {"energy": e[0], "forces": f[:n], "stress": s,
                "local_var": v[:n], "latency_ms": lat.value}

    def result(self, rid, timeout=600.0):
        t0 = time.time()
        while True:
            r = self.poll(rid)
            if r is not None:
                return r
            if time.time() - t0 > timeout:
                raise TimeoutError(f"request {rid} not done after {timeout} s")
            time.sleep(0.0005)

    def stats(self):
        c, b, bpa = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().fgb_serve_stats(self.h, ctypes.byref(c), ctypes.byref(b),
                                    ctypes.byref(bpa)))
        return {"completed": c.value, "batches": b.value,
                "bytes_per_atom": bpa.value}

    def close(self):
        if getattr(self, "h", None) is not None:
            lib().fgb_serve_stop(self.h)
            self.h = None

    def __del__(self):
        if _lib._lib is not None:
            self.close()
