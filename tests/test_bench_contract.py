"""bench.py's CPU-side contract: the traffic figures its roofline objects read
from the profile summaries, and the reference arm's JSON line (the reference
algorithm timed on the host cores; no GPU)."""
import json
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _traffic_keys():
    src = open(os.path.join(ROOT, "bench.py")).read()
    return sorted(set(re.findall(r'profile_traffic\("([A-Za-z0-9_]+)"\)', src)))


def test_every_traffic_key_is_recorded_in_a_profile():
    keys = _traffic_keys()
    assert keys, "bench.py reads no traffic figure"
    for k in keys:
        v = bench.profile_traffic(k)
        assert isinstance(v, int) and v > 0, k


def test_profile_traffic_parses_only_its_line_form(tmp_path, monkeypatch):
    (tmp_path / "profiles").mkdir()
    (tmp_path / "profiles" / "x.md").write_text(
        "prose traffic[k1] = 5 bytes (not at the start of a line)\n"
        "traffic[k2] = 1,000 bytes (commas are not a number)\n"
        "  traffic[k3] = 4096 bytes per launch\n")
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.profile_traffic("k1") is None
    assert bench.profile_traffic("k2") is None
    assert bench.profile_traffic("k3") == 4096
    assert bench.profile_traffic("absent") is None


def test_workload_config_is_shared_by_both_arms():
    c1, c2 = bench.workload_config(1), bench.workload_config(2)
    assert set(c1) == set(c2) == {"workload", "batch_per_gpu", "global_batch", "l2", "parallelism"}
    assert c1["global_batch"] == bench.BATCH and c2["global_batch"] == 2 * bench.BATCH


@pytest.mark.timeout(300)
def test_reference_arm_prints_one_contract_line():
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=280, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["config"] == bench.workload_config(1)
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert isinstance(cb["sample"], str) and cb["sample"]


def _profile_commands():
    cmds = []
    for f in sorted(os.listdir(os.path.join(ROOT, "profiles"))):
        if f.endswith((".md", ".txt")):
            for line in open(os.path.join(ROOT, "profiles", f)):
                for m in re.finditer(r"python ([A-Za-z_]+\.py)((?: [^&|>\\\n]*)?)", line):
                    cmds.append((f, m.group(1), m.group(2).split()))
    return cmds


def test_profile_commands_run_committed_files():
    """Every command a profile summary gives runs a committed script with a
    case and flags that script accepts."""
    import bench_cases

    cmds = _profile_commands()
    assert cmds
    bench_flags = {"--gpus", "--steps", "--warmup", "--impl", "--headline-only"}
    for f, script, args in cmds:
        assert os.path.exists(os.path.join(ROOT, script)), (f, script)
        if script == "bench_cases.py":
            assert args and args[0] in bench_cases.CASES, (f, args)
            assert {a for a in args[1:] if a.startswith("--")} <= {"--reps", "--variant"}, (f, args)
        elif script == "bench.py":
            assert {a for a in args if a.startswith("--")} <= bench_flags, (f, args)
    src = open(os.path.join(ROOT, "bench.py")).read()
    for flag in bench_flags:
        assert f'"{flag}"' in src, flag
