"""Host side of the tile-shape autotuner: the candidate list and the JSON
cache (path override, atomic round trip, unreadable files).  CPU only."""
import json

from pylians3_gb300 import autotune


def test_candidates_fit_the_grid():
    for dims in (16, 64, 512):
        c = autotune.candidates(dims)
        assert c and all(max(s) <= max(8, dims) for s in c)
        assert all(tz in (16, 32) and tx in (8, 16, 32) and ty in (8, 16, 32) for tx, ty, tz in c)
    assert len(autotune.candidates(512)) == 18


def test_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("PYLGPU_TUNE_CACHE", str(path))
    assert autotune.cache_path() == str(path)
    assert autotune._read_cache() == {}                      # no file yet
    entry = {"GB300|256|CIC|24|0": {"shape": [16, 32, 32, 64], "ms": 0.24,
                                    "default": [16, 32, 32, 32], "default_ms": 0.25}}
    autotune._write_cache(entry)
    assert json.loads(path.read_text()) == entry
    assert autotune._read_cache() == entry
    assert not [p for p in tmp_path.iterdir() if ".tmp" in p.name]   # replaced atomically


def test_unreadable_cache_is_empty(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    monkeypatch.setenv("PYLGPU_TUNE_CACHE", str(path))
    assert autotune._read_cache() == {}
