"""GPU: the tcgen05 and TMA properties the exact-slicing GEMM is designed
around, re-measured by small probes under tests/probes (each compiled with
nvcc for sm_103a and run once): an M = 128 MMA costs max(64, N/2) cycles,
the 13 stacked-N MMAs of a k-step run near the tensor peak, and two bulk
copies per chunk feed the ring faster than eighteen."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def run_probe(name, tmp_path):
    exe = str(tmp_path / name)
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-O3", "-std=c++17", "-o", exe,
                    os.path.join(HERE, "probes", name + ".cu")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True,
                         text=True, timeout=120).stdout
    print(out)
    assert "err=1" not in out and "cuda=0" in out
    return out


def test_mma_cost_and_span_plan(tmp_path):
    out = run_probe("tcgen05_mma_cost", tmp_path)
    cyc = {int(n): float(c) for n, c in
           re.findall(r"N=\s*(\d+) rotate=0 reps=\d+: issue [\d.]+ cyc/mma, "
                      r"complete ([\d.]+)", out)}
    assert cyc[48] > 55 and cyc[128] < 70 and 120 < cyc[256] < 140
    plan = dict(re.findall(r"plan (.+?): ([\d.]+) cyc per k-step", out))
    assert float(plan["13 spans"]) < 0.45 * float(plan["45 x N=48"])


def test_load_ring_chunk_major(tmp_path):
    out = run_probe("ozaki_load_ring", tmp_path)
    cyc = {(int(s), int(m), int(c)): float(v) for s, m, c, v in
           re.findall(r"stages=(\d) mma=(\d) chunk_major=(\d): [\d.]+ ms, "
                      r"(\d+) cycles", out)}
    assert cyc[(4, 0, 1)] < 0.6 * cyc[(4, 0, 0)]
    assert cyc[(4, 1, 1)] < cyc[(4, 1, 0)]


def test_tmem_drain(tmp_path):
    out = run_probe("tmem_drain", tmp_path)
    assert "mode 0:" in out and "mode 2:" in out


def test_fp32_and_double_float_throughput(tmp_path):
    """FP32 FMA and double-float multiply-accumulate throughput of the SMs:
    the bounds the double-float descriptor stage is measured against."""
    out = run_probe("fp32_peak", tmp_path)
    m = re.search(r"fp32_tflops=([\d.]+) dfmac_gops=([\d.]+)", out)
    fp32, dfmac = float(m.group(1)), float(m.group(2))
    assert fp32 > 30.0 and dfmac > 500.0, out
