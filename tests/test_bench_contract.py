"""The bench's reference arm (`bench.py --impl reference`) on the CPU.

It times the reference's algorithm (the oracle, one process per host core)
on the bench's workloads and prints one JSON line with the contract's keys;
under a distributed launch only rank 0 runs and prints.  These runs need no
GPU, so they are checked here with one short step."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, env=None):
    e = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        e.pop(k, None)
    e.update(env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, env=e,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout


def _line(out):
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out[-2000:]
    return json.loads(lines[0])


def _check_common(d):
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["unit"] == "solves/s" and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["vs_baseline"] is None
    cb = d["cpu_baseline"]
    assert set(cb) >= {"value", "unit", "cores", "kind", "sample"}
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_single_instance_line():
    d = _line(_run(["--workload", "portfolio_n100_fp64", "--impl", "reference", "--steps", "2",
                    "--warmup", "1"]))
    _check_common(d)
    assert d["metric"].startswith("solves/s at EPS_ABS 0.005")
    assert d["steps"] == 2 and d["warmup"] == 1
    assert d["config"]["workload"] == "portfolio_n100_fp64"


def test_reference_arm_batch_line():
    d = _line(_run(["--impl", "reference", "--steps", "1", "--warmup", "0"]))
    _check_common(d)
    assert d["metric"].startswith("solves/s at EPS_ABS 1e-4: batched + learned warm start")
    assert d["config"]["workload"] == "portfolio_family_warmstart"
    assert d["cpu_baseline"]["cores"] == (os.cpu_count() or 1)


def test_reference_arm_other_ranks_print_nothing():
    out = _run(["--impl", "reference", "--steps", "1", "--warmup", "0"],
               env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert not [l for l in out.splitlines() if l.startswith("{")]


def test_reference_arm_uneven_full_is_bounded():
    """The full-size uneven batch: a stratified subsample (here 2 instances
    per n-decile), a few ADMM iterations each, extrapolated (a full reference
    solve of the largest instances takes minutes)."""
    d = _line(_run(["--workload", "portfolio_uneven_full", "--impl", "reference", "--steps", "1",
                    "--warmup", "0", "--batch", "64", "--cpu-per-decile", "2"]))
    _check_common(d)
    assert d["metric"].startswith("solves/s at EPS_ABS 1e-4: batched uneven instances")
    assert d["config"]["workload"] == "portfolio_uneven_full"
    assert d["config"]["instances_per_step"] == 64
    assert "stratified subsample of 20 instances" in d["cpu_baseline"]["sample"]
