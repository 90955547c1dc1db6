"""bench.py on the CPU: the helpers behind the CPU baseline, the mixed-solve
case table, and the reference arm's JSON line (the reference arm runs the
oracle on the host cores, so it needs no GPU)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


@pytest.mark.parametrize("n", [64, 100, 512, 8192])
def test_step_flops_sum_to_the_blocked_lu(n):
    steps = -(-n // bench.NB)
    total = sum(bench.lu_step_flops(n, b) for b in range(steps))
    assert total == pytest.approx(bench.lu_block_flops(n), rel=1e-12)
    # the blocked count is the textbook 2/3 n^3 to leading order
    if n >= 512:
        assert total == pytest.approx(2.0 * n ** 3 / 3.0, rel=0.02)


def test_sample_blocks_spread_over_the_factorisation():
    assert bench.lu_sample_blocks(8192) == [0, 32, 64, 96, 120]
    for n in (64, 100, 1000, 16384):
        blocks = bench.lu_sample_blocks(n)
        assert blocks == sorted(set(blocks))
        assert 0 in blocks and max(blocks) < -(-n // bench.NB)


def test_seconds_from_constant_rates():
    n, rate = 4096, 2.5e9
    rates = {b: rate for b in bench.lu_sample_blocks(n)}
    want = (bench.lu_block_flops(n) + 2.0 * n * n) / rate
    assert bench.lu_seconds_from_samples(n, rates) == pytest.approx(want, rel=1e-12)


def test_seconds_interpolate_between_samples():
    # rate 1 at step 0, 3 at the last sample: every step between gets a rate
    # in [1, 3], so the total lies between the two constant-rate totals
    n = 2048
    blocks = bench.lu_sample_blocks(n)
    rates = {b: 1.0 + 2.0 * b / blocks[-1] for b in blocks}
    t = bench.lu_seconds_from_samples(n, rates)
    flops = bench.lu_block_flops(n) + 2.0 * n * n
    assert flops / 3.0 < t < flops / 1.0


def test_mixed_cases_table():
    labels = [(k, r, lab) for k, r, lab, *_ in bench.MIXED_CASES]
    assert len(labels) == len(set(labels))
    for kappa, nrhs, label, prec, solver, max_iter in bench.MIXED_CASES:
        assert kappa in (1e2, 1e6, 1e10) and nrhs in (1, 64)
        assert prec in (0, 1, 2, 3, 4, 5, 6) and solver in (0, 1, 2) and max_iter > 0
    # every factor precision the configuration names is measured at kappa = 1e2
    precs = {p for k, _, _, p, _, _ in bench.MIXED_CASES if k == 1e2}
    assert {1, 2, 3, 4, 6} <= precs
    # kappa = 1e10 is measured, and met by FP64-accurate factors
    assert any(k == 1e10 and p == 4 for k, _, _, p, _, _ in bench.MIXED_CASES)


def test_reference_arm_json_line():
    # a small n keeps the oracle's block steps short; the line's contract is
    # the same as at the benchmark's n = 8192
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--n", "512", "--steps", "2", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "solves/s"
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] == 3
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0
    assert e2e["d2h_bytes_per_step"] == 0
