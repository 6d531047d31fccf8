"""bench.py's host helpers on the CPU: the per-launch DRAM traffic that the
roofline object takes from the committed ncu summaries, and the summaries'
own hygiene (each names its kernel and workload, gives the ncu command it
came from, and that command leaves the GPU clocks alone)."""
import importlib.util
import re
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    argv, sys.argv = sys.argv, ["bench.py"]
    try:
        spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
    finally:
        sys.argv = argv
    return m


# (kernel, workload, algorithmic bytes per interior point and shot, points)
CASES = [
    ("k_vd_v + k_vd_p<corr> adjoint", "acoustic_vd2d_2001x801", 68 + 12 / 8, 1999 * 799),
]


@pytest.mark.parametrize("kernel,workload,bpp,pts", CASES)
def test_traffic_lookup_matches_algorithmic_bytes(bench, kernel, workload, bpp, pts):
    """DRAM bytes per launch and shot are found and lie within [0.5, 1.3] of the
    algorithmic bytes (below 1 where the small capture's L2 still holds part
    of the previous step; above 1 would mean re-reads)."""
    t = bench._traffic_from_profiles(kernel, workload)
    assert t is not None and t > 0
    assert 0.5 <= t / (bpp * pts) <= 1.3, t / (bpp * pts)


def test_traffic_lookup_unknown_kernel(bench):
    assert bench._traffic_from_profiles("k_no_such_kernel", "acoustic2d_2001x801") is None
    assert bench._traffic_from_profiles("k_ac2d_step<3>", "no_such_workload") is None


@pytest.mark.parametrize("kind", ["recompute", "adjoint"])
def test_traffic_ratio_of_the_2d_kinds(bench, kind):
    """The 2D gradient kinds' DRAM/algorithmic ratio comes from the committed
    16-shot capture: below 1 (no re-reads), above 0.5."""
    r = bench._traffic_ratio_from_profiles(kind, "acoustic2d_2001x801")
    assert r is not None and 0.5 <= r <= 1.05, r


def test_traffic_ratio_unknown(bench):
    assert bench._traffic_ratio_from_profiles("forward", "acoustic2d_2001x801") is None
    assert bench._traffic_ratio_from_profiles("adjoint", "no_such_workload") is None


def test_profile_summaries_name_their_command():
    files = sorted((ROOT / "profiles").glob("*.md"))
    assert files
    for f in files:
        txt = f.read_text()
        cmds = [ln for ln in txt.splitlines() if re.match(r"\s*ncu\s", ln)]
        assert cmds, f"{f.name}: no ncu command"
        for c in cmds:
            assert "--clock-control none" in c, f"{f.name}: {c.strip()}"
        assert "bench.py" in txt, f.name


def _run_bench(args, env_extra=None):
    import json
    import os
    import subprocess
    env = dict(os.environ, **(env_extra or {}))
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True, env=env,
                       timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_json_line():
    """bench.py --impl reference (the oracle port on the host cores) prints one
    JSON line with the contract's keys on a bounded sample."""
    out = _run_bench(["--impl", "reference", "--workload", "acoustic2d_201", "--steps", "1", "--warmup", "0",
                      "--cpu-sample-nt", "20"])
    assert len(out) == 1
    d = out[0]
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "Gpts/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]


def test_reference_arm_other_ranks_do_no_work():
    """Under torchrun only rank 0 runs the reference arm; the others exit 0 silently."""
    out = _run_bench(["--impl", "reference", "--workload", "acoustic2d_201", "--steps", "1", "--warmup", "0",
                      "--cpu-sample-nt", "20"], {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert out == []
