"""CPU: the autotuner's host-side state (tune.cu) — the FGB_TUNE_CACHE file
is read once per process, keeping only the lines of this device (the
device tag is "unknown" without a GPU), and the force / clear / entry calls
validate their arguments.  Runs in a fresh process for a clean state."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import ctypes, os, sys
sys.path.insert(0, os.environ["FGB_ROOT"])
from flare_gb300 import _lib
L = _lib.lib()
assert L.fgb_tune_set_mode(1) == 0          # first use: reads the cache file
assert L.fgb_tune_count() == 2, L.fgb_tune_count()
key = (ctypes.c_int * 5)()
ms = (ctypes.c_double * 4)()
seen = []
for i in range(2):
    assert L.fgb_tune_entry(i, key, ms) == 0
    seen.append(tuple(key))
assert seen == [(0, 16384, 1000, 680, 2), (1, 16384, 1000, 1000, 0)], seen
assert L.fgb_tune_entry(2, key, ms) == _lib.FGB_EINVAL
assert L.fgb_tune_force(0, 1) == 0 and L.fgb_tune_force(0, -1) == 0
assert L.fgb_tune_force(7, 0) == _lib.FGB_EINVAL
assert L.fgb_tune_force(0, 9) == _lib.FGB_EINVAL
assert L.fgb_tune_set_mode(2) == _lib.FGB_EINVAL
assert L.fgb_tune_clear() == 0 and L.fgb_tune_count() == 0
print("ok")
"""


def test_tune_cache_file_and_arguments(tmp_path):
    cache = tmp_path / "tune.txt"
    cache.write_text("unknown 0 16384 1000 680 2\n"
                     "GB300|152 0 16384 1000 680 1\n"     # another device
                     "unknown 1 16384 1000 1000 0\n"
                     "unknown 0 1 2 3 9\n"                 # bad candidate
                     "unknown 5 1 2 3 0\n")                # bad operation
    script = tmp_path / "t.py"
    script.write_text(SCRIPT)
    env = dict(os.environ, FGB_ROOT=ROOT, FGB_TUNE_CACHE=str(cache),
               CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, str(script)], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr
