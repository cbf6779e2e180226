"""The integer-pipe FP64 running sum of the exact row sums
(spacelab_gb300/csrc/sl_sum_exact.cuh), checked on the host against IEEE
double additions: single additions in right and wrong frames (random,
cancelling, halfway, few-bit and special operands) and whole 5000-term rows
summed in 16-term chunks with the FP64 repeat of failed chunks, as the GPU
kernel sums them.  The GPU side is tests/test_gpu_parity.py's
test_rowsum_methods_bit_identical."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_integer_pipe_sum_matches_ieee_additions(tmp_path):
    exe = tmp_path / "sum_exact_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-Werror",
                    "-I", str(ROOT / "spacelab_gb300" / "csrc"), str(ROOT / "tests" / "sum_exact_check.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "2000000", "300"], stdout=subprocess.PIPE, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    stats = {line.split()[0]: line.split() for line in out.stdout.splitlines() if line.strip()}
    pairs = stats["pairs"]
    assert int(pairs[3]) > 1_000_000, out.stdout  # the fast path is exercised, not only the fallback
    chunks = stats["chunks"]
    assert int(chunks[3]) < int(chunks[1]) // 5, out.stdout
    assert stats["mismatches"][1] == "0", out.stdout
