"""Tile-shape autotuner of the sliced tensor-core GEMMs (``fgb_tune_*``).

The kernel, variance and force GEMMs of the mixed-precision path each have
a few candidate tile shapes with identical results; the fastest is timed and
chosen per problem shape at first use.  ``FGB_TUNE_CACHE=<file>`` keeps the
choices across processes, ``FGB_AUTOTUNE=0`` starts with tuning off.
"""
import numpy as np

from ._lib import check, lib, ptr

OPS = ("kernel_gemm", "variance_gemm", "force_gemm")
CANDIDATES = {
    "kernel_gemm": ("B tile 48 rows", "B tile 32 rows",
                    "B tile 64 rows (8 or 7 slices)"),
    "variance_gemm": ("B tile 48 rows", "B tile 32 rows",
                      "B tile 64 rows (8 or 7 slices)"),
    "force_gemm": ("B tile 128 rows, 2 epilogue warps",
                   "B tile 128 rows, 4 epilogue warps",
                   "B tile 64 rows, 2 epilogue warps"),
}


def set_mode(tune=True):
    """Tune at first use (True, the default) or always take candidate 0."""
    check(lib().fgb_tune_set_mode(1 if tune else 0), "autotune.set_mode")


def force(op, candidate):
    """Pin operation ``op`` (a name of OPS) to ``candidate`` (None: tune)."""
    c = -1 if candidate is None else int(candidate)
    check(lib().fgb_tune_force(OPS.index(op), c), "autotune.force")


def clear():
    """Forget every tuned shape."""
    check(lib().fgb_tune_clear(), "autotune.clear")


def table():
    """Tuned shapes: op, rows bucket, columns, depth, chosen candidate and
    the best timed launch (ms) of each candidate."""
    out = []
    key = np.zeros(5, np.int32)
    ms = np.zeros(4, np.float64)
    for i in range(lib().fgb_tune_count()):
        check(lib().fgb_tune_entry(i, ptr(key), ptr(ms)), "autotune.table")
        op = OPS[int(key[0])]
        n = len(CANDIDATES[op])
        out.append({"op": op, "rows_bucket": int(key[1]),
                    "cols": int(key[2]), "depth": int(key[3]),
                    "choice": int(key[4]),
                    "choice_shape": CANDIDATES[op][int(key[4])],
                    "ms": [float(x) for x in ms[:n]]})
    return out


__all__ = ["OPS", "CANDIDATES", "set_mode", "force", "clear", "table"]
