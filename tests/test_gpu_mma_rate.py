"""tcgen05.mma issue rate on one SM (tests/mma_rate.cu), the measurement the
fixed-point GEMM's tile widths rest on: an M = 128, K = 16 MMA with bf16
operands in shared memory runs at the full 8192 FP32-accumulate operations per
cycle from N = 128 up, while narrower MMAs take at least ~46 cycles, about the
time to read A (4 KB) and B (N x 32 B) from shared memory at 128 B per cycle.
Two accumulators taken in turn cost nothing over one."""
import json
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_mma_rate(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "mma_rate")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-o", exe,
                    os.path.join(HERE, "mma_rate.cu")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120).stdout
    rows = {(r["mode"], r["n"]): r for r in json.loads(out)["rows"]}
    print(json.dumps(list(rows.values())))
    for n in (128, 192, 256):
        assert rows[(0, n)]["efficiency"] > 0.9
    # narrow MMAs are bounded by a floor of tens of cycles, not by their width
    assert rows[(0, 16)]["cycles_per_mma"] > 30
    # alternating two accumulators runs at the single-accumulator rate
    assert rows[(1, 80)]["cycles_per_mma"] < 1.1 * rows[(0, 80)]["cycles_per_mma"]
