"""The autotuner's search and its hand-off to the build, on the CPU (the
timings come from a stand-in; GPU runs time real builds)."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "sph-mesh-generation_gb300"))
from mrsph import autotune, build  # noqa: E402


def test_coordinate_search_finds_separable_minimum():
    target = {"A": 3, "B": 1, "C": 7}
    space = {"A": [1, 2, 3], "B": [0, 1, 2], "C": [5, 7]}
    calls = []

    def timer(s):
        calls.append(dict(s))
        return sum(abs(s[k] - target[k]) for k in target) + 1.0

    best, t, tried = autotune.coordinate_search(timer, {"A": 1, "B": 2, "C": 5}, space, log=lambda *_: None)
    assert best == target and t == 1.0
    assert len(calls) == len({tuple(sorted(c.items())) for c in calls}) == len(tried)


def test_defaults_are_in_the_space():
    for k, v in autotune.DEFAULTS.items():
        assert v in autotune.SPACE[k], k
    assert autotune.defines_of({"TILE_UNROLL": 4}) == ["-DMRSPH_TILE_UNROLL=4"]


def test_build_reads_tuned_file(tmp_path, monkeypatch):
    monkeypatch.delenv("MRSPH_NVCC_DEFINES", raising=False)
    f = tmp_path / "tuned.json"
    f.write_text(json.dumps({"defines": {"TILE_SPAN_X": 5, "DENSITY_MIN_BLOCKS": 5}}))
    monkeypatch.setattr(build, "TUNED", str(f))
    assert build.tuned_defines() == ["-DMRSPH_DENSITY_MIN_BLOCKS=5", "-DMRSPH_TILE_SPAN_X=5"]
    monkeypatch.setenv("MRSPH_NVCC_DEFINES", "-DMRSPH_TILE_UNROLL=2")
    assert build.tuned_defines() == ["-DMRSPH_TILE_UNROLL=2"]
    monkeypatch.setattr(build, "TUNED", str(tmp_path / "absent.json"))
    monkeypatch.delenv("MRSPH_NVCC_DEFINES")
    assert build.tuned_defines() == []
