"""bench.py's reference arm (CPU): one JSON line with the contract's keys —
impl, the headline metric and unit, higher_is_better, a cpu_baseline that
describes the run (kind, cores, sample) and an e2e object with no
host-device bytes — from the CPU restatement on a small sample."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_line():
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--cpu-seconds", "1"], capture_output=True, text=True, timeout=300,
                         cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "Msamples/s at 1080p" and d["unit"] == "Msamples/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert d["config"]["resolution"] == "1920x1080"


def test_relmse_crossing_time():
    sys.path.insert(0, str(ROOT))
    import bench
    # relMSE falling as 1/time: the crossing of 1e-3 is at exactly 2 s
    curve = [(0.5, 16, 4e-3), (1.0, 32, 2e-3), (4.0, 128, 5e-4)]
    t, reached = bench.crossing_time(curve, 1e-3)
    assert reached and abs(t - 2.0) < 1e-9
    # below the target at the first reading
    assert bench.crossing_time([(0.3, 16, 5e-4)], 1e-3) == (0.3, True)
    # never reached: extrapolated as relMSE ~ 1/time
    t, reached = bench.crossing_time([(1.0, 16, 4e-3), (2.0, 32, 2e-3)], 1e-3)
    assert not reached and abs(t - 4.0) < 1e-9


def test_profile_figures_only_for_the_current_build(tmp_path, monkeypatch):
    """bench.py quotes ncu counters from a committed profile summary only
    when that capture was taken of the current kernel sources."""
    sys.path.insert(0, str(ROOT))
    import bench
    h = bench.source_hash()
    assert h == bench.source_hash() and len(h) == 16
    assert bench.source_hash(bench.MEGA_SOURCES) != h
    prof = tmp_path / "profiles"
    prof.mkdir()
    fig = {"sources": h, "dram_bytes_per_visit": 1.5, "l1tex_pct": 60.0}
    (prof / "k_now.md").write_text("# k\n\nfigures: " + json.dumps(fig) + "\n")
    (prof / "k_old.md").write_text("figures: " + json.dumps(dict(fig, sources="0" * 16)) + "\n")
    (prof / "k_none.md").write_text("# no figures\n")
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    monkeypatch.setattr(bench, "source_hash", lambda files=None: h)
    d, src = bench.profile_figures("k_now")
    assert d["dram_bytes_per_visit"] == 1.5 and "this build" in src
    assert bench.profile_figures("k_old")[0] is None
    assert bench.profile_figures("k_none")[0] is None
    assert bench.profile_figures("k_absent")[0] is None


def test_port_speed_record():
    """The restatement's speed against the reference's own kernels (same
    flags, same cores), measured where the reference sources are."""
    d = json.loads((ROOT / "oracle" / "port_speed.json").read_text())
    assert d["accumulation_bit_identical"] is True
    assert "-O3" in d["flags"] and "-ffp-contract=off" in d["flags"]
    for k in ("all_threads", "one_thread"):
        assert d["restatement_over_reference"][k] > 0
