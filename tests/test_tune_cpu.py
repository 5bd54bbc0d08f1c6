"""The autotuner's cache on CPU: cached shapes are answered without timing,
keys separate operations and shapes, and a missing, corrupt or unwritable
cache file costs only the cache (timing itself needs a GPU and is covered by
the GPU tests)."""

from __future__ import annotations

import json

import pytest

from voxelproj_gb300 import tune


@pytest.fixture
def cache_file(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("VOXELPROJ_GB300_TUNE_CACHE", str(path))

    def no_timing(*_a, **_k):
        raise AssertionError("a cached shape must not be timed")

    monkeypatch.setattr(tune, "_time", no_timing)
    return path


def test_cache_path_follows_environment(cache_file):
    assert tune.cache_path() == cache_file


def test_cached_batch_variant_is_not_timed(cache_file):
    cache_file.write_text(json.dumps({
        "batch/forward/z0/96x96x96/px96": {"variant": 11, "ms": {"10": 1.0, "11": 0.5}},
        "batch/backward/z0/96x96x96/px96": {"variant": 6, "ms": {"7": 2.0, "6": 1.0}},
    }))
    assert tune.batch_variant("forward", 96, 300) == 11
    assert tune.batch_variant("backward", 96, 45) == 6  # angle count is not in the key


def test_cached_single_variant_keys_by_shape(cache_file):
    cache_file.write_text(json.dumps({
        "single/forward/z0/64x64x128/90x64x128": {"variant": 13, "ms": {}},
        "single/forward/z0/64x64x256/90x64x256": {"variant": 10, "ms": {}},
    }))
    assert tune.tune_single("forward", (64, 64, 128), (90, 64, 128), apply=False) == 13
    assert tune.tune_single("forward", (64, 64, 256), (90, 64, 256), apply=False) == 10


def test_corrupt_cache_reads_as_empty(cache_file):
    cache_file.write_text("{not json")
    assert tune._load() == {}


def test_missing_cache_reads_as_empty(cache_file):
    assert not cache_file.exists()
    assert tune._load() == {}


def test_store_round_trips_and_replaces_atomically(cache_file):
    tune._store({"k": {"variant": 7, "ms": {"7": 1.5}}})
    assert json.loads(cache_file.read_text()) == {"k": {"variant": 7, "ms": {"7": 1.5}}}
    assert not cache_file.with_suffix(".tmp").exists()
    tune._store({"k": {"variant": 6, "ms": {}}})
    assert tune._load()["k"]["variant"] == 6


def test_unwritable_cache_is_ignored(tmp_path, monkeypatch):
    blocker = tmp_path / "file"
    blocker.write_text("")
    # the cache's directory would have to be a regular file: storing fails
    monkeypatch.setenv("VOXELPROJ_GB300_TUNE_CACHE", str(blocker / "sub" / "tune.json"))
    tune._store({"k": {"variant": 1}})  # no exception
    assert tune._load() == {}
