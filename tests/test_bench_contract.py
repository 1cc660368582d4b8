"""The benchmark's contract on the CPU: the reference arm's JSON line (the
oracle's OpenMP PCGPME timed on the host cores, no GPU needed) and the fixed
counts the rooflines divide by."""
import json
import subprocess
import sys

import pytest

import __graft_entry__ as ge

ROOT = ge.ROOT


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "tank_64x64x32",
                          "--steps", "1", "--warmup", "1"], cwd=ROOT, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "pressure solves/s" and line["unit"] == "solves/s"
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["config"]["workload"] == "tank_64x64x32" and line["config"]["rows"] == 86016
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "solves/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_roofline_counts():
    """Algorithmic bytes per row: 62 words of setup and 68 per iteration (the
    streams of one operator application are 25 words: AXSUB 9, sweeps 1-4 12,
    sweep 5/6 4; an iteration adds 18 words of vector passes); FP64 work: 37
    fused multiply-adds per row and iteration (AXSUB 7 and LDUSUB 6 per
    application, RQ, e, AMU and SS, x, r, RN and C1, p: 11)."""
    sys.path.insert(0, str(ROOT))
    import bench
    n, it = 1000, 100
    assert bench.bytes_solve_fp64(n, it) == n * 8 * (62 + 68 * it)
    assert bench.bytes_solve_mixed(n, 300, 7) == n * (96 + 4 * 62 * 7 + 4 * 68 * 300 + 100 * 7)
    assert bench.bytes_solve_fp64_with_indices(n, it) - bench.bytes_solve_fp64(n, it) == n * (72 + 96 * it)
    per_application = 7 + 6
    assert bench.FMA_ROW_ITER_FP64 == 2 * per_application + 1 + 1 + 2 + 2 + 1 + 2 + 2
