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
    ("k_ac2d_step<3>", "acoustic2d_2001x801", 28 + 4 / 8, 1999 * 799),
    ("k_ac2d_step<1> recompute", "acoustic2d_2001x801", 20 + 4 / 8, 1999 * 799),
    ("k_ac2d_step<0>", "acoustic2d_2001x801", 16 + 4 / 8, 1999 * 799),
    ("k_ac2d_adj_grp", "acoustic2d_2001x801", 24 + 4 / 8, 1999 * 799),
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
