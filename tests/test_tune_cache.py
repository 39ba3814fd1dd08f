"""Host logic of the autotuners' JSON cache files (csrc/tune_cache.cpp,
used by orn_batch_tune and orn_wave_tune): compiled here with a small
driver and checked on files holding both tuners' entries, hand edits and
damaged entries."""
import json
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parent.parent / "zig_ornament_gb300" / "csrc"

DRIVER = r"""
#include "tune_cache.h"
#include <cstdio>
// read argv[1], print every entry, add/replace entry argv[3] (shape/fetch/steps
// 1/8/64, 2.5 ms) and write the result to argv[2]
int main(int argc, char** argv) {
    if (argc < 4) return 2;
    auto m = orn::read_tune_cache(argv[1]);
    for (const auto& kv : m) {
        std::printf("%s|%.3f", kv.first.c_str(), kv.second.ms);
        for (const auto& f : kv.second.fields) std::printf("|%s=%ld", f.first.c_str(), f.second);
        std::printf("\n");
    }
    orn::TuneEntry e;
    e.fields["shape"] = 1;
    e.fields["fetch"] = 8;
    e.fields["steps"] = 64;
    e.ms = 2.5;
    m[argv[3]] = e;
    return orn::write_tune_cache(argv[2], m, {"shape", "fetch", "steps"}) ? 0 : 1;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("tune_cache")
    (d / "t.cpp").write_text(DRIVER)
    exe = d / "t"
    subprocess.run(["g++", "-std=c++17", f"-I{CSRC}", str(d / "t.cpp"), str(CSRC / "tune_cache.cpp"), "-o", str(exe)],
                   check=True)
    return exe


def run(driver, src, dst, key):
    out = subprocess.run([str(driver), str(src), str(dst), key], check=True, capture_output=True, text=True).stdout
    rows = {}
    for line in out.splitlines():
        parts = line.split("|")
        # keys hold '|' themselves: the last fields are ms and name=value pairs
        i = next(k for k in range(len(parts)) if "=" not in parts[k] and k > 0 and
                 all("=" in p for p in parts[k + 1:]))
        rows["|".join(parts[:i])] = (float(parts[i]), dict(p.split("=") for p in parts[i + 1:]))
    return rows


def test_round_trip_keeps_both_tuners_entries(driver, tmp_path):
    src = tmp_path / "in.json"
    src.write_text(json.dumps({
        "GB300|sm152|scenes=64|pixels=58517504": {"block": 64, "blocks_per_sm": 8, "shade_threshold": 4,
                                                  "ms": 5496.397},
        "GB300|sm152|wavefront|pixels=2073600": {"shape": 0, "fetch": 4, "steps": 32, "ms": 47.25}}, indent=1))
    dst = tmp_path / "out.json"
    rows = run(driver, src, dst, "new|key")
    assert rows["GB300|sm152|scenes=64|pixels=58517504"] == (
        5496.397, {"block": "64", "blocks_per_sm": "8", "shade_threshold": "4"})
    assert rows["GB300|sm152|wavefront|pixels=2073600"] == (47.25, {"shape": "0", "fetch": "4", "steps": "32"})
    data = json.loads(dst.read_text())
    assert data["GB300|sm152|scenes=64|pixels=58517504"] == {"block": 64, "blocks_per_sm": 8,
                                                             "shade_threshold": 4, "ms": 5496.397}
    assert data["GB300|sm152|wavefront|pixels=2073600"] == {"shape": 0, "fetch": 4, "steps": 32, "ms": 47.25}
    assert data["new|key"] == {"shape": 1, "fetch": 8, "steps": 64, "ms": 2.5}
    # the written file reads back the same
    assert run(driver, dst, tmp_path / "again.json", "new|key") == run(driver, dst, tmp_path / "x.json", "new|key")


def test_missing_and_damaged_files(driver, tmp_path):
    dst = tmp_path / "out.json"
    assert run(driver, tmp_path / "absent.json", dst, "k") == {}
    assert json.loads(dst.read_text()) == {"k": {"shape": 1, "fetch": 8, "steps": 64, "ms": 2.5}}
    bad = tmp_path / "bad.json"
    bad.write_text('{"a": {"shape": 2, "fetch": }, "b": 3, "c": {"steps": 64, "ms": 1.0}, "d": {"shape": 1')
    rows = run(driver, bad, tmp_path / "out2.json", "k")
    # an entry keeps only the fields that parse; the tuners re-tune entries
    # that miss one of theirs
    assert rows["a"][1] == {"shape": "2"}
    assert rows["c"] == (1.0, {"steps": "64"})
    assert "b" not in rows and "d" not in rows
