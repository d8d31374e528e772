"""The autotuner's host side: choices are keyed by workload shape and a
cached choice (from its JSON file or from memory) comes back without any
timing run."""
import json

import numpy as np
import pytest


def _autotune():
    try:
        from libnabo_gb300 import autotune
    except Exception as e:  # noqa: BLE001 -- the package needs its built library
        pytest.skip(f"package not importable: {e}")
    return autotune


def test_shape_key():
    A = _autotune()
    assert A.shape_key([1000, 3000], 3, np.float32, [5, 16]) == "d3-float32-k16-n2^11"
    assert A.shape_key([40], 8, np.float64, [1]) == "d8-float64-k1-n2^5"
    # the mean size, rounded to a power of two, is what distinguishes batches
    assert A.shape_key([1000, 1100], 3, np.float32, 10) == A.shape_key([1050], 3, np.float32, 10)


def test_cached_choice_needs_no_timing(tmp_path):
    A = _autotune()
    clouds = [np.zeros((1000, 3), np.float32), np.zeros((3000, 3), np.float32)]
    queries = [c[:10] for c in clouds]
    key = A.shape_key([1000, 3000], 3, np.float32, [5, 16])
    path = tmp_path / "tune.json"
    stored = {"bucketSize": 12, "threadsPerBlock": 64, "maxLevels": 30, "sample_ms": 1.5}
    path.write_text(json.dumps({key: stored}))
    A._cache.clear()
    got = A.tune(clouds, queries, [5, 16], cache_path=str(path))
    assert got["cached"] and got["key"] == key
    assert {k: got[k] for k in stored} == stored
    again = A.tune(clouds, queries, [5, 16])  # now from memory, no file
    assert again["cached"] and again["bucketSize"] == 12
    A._cache.clear()


def test_restricted_candidates_are_cached_under_their_own_key(tmp_path):
    """A tuning restricted to some split rules or lanes per query is stored
    apart from the unrestricted one (a restricted run must not answer an
    unrestricted request, nor the reverse)."""
    A = _autotune()
    clouds = [np.zeros((1000, 8), np.float32), np.zeros((3000, 8), np.float32)]
    queries = [c[:10] for c in clouds]
    base = A.shape_key([1000, 3000], 8, np.float32, 32)
    path = tmp_path / "tune.json"
    path.write_text(json.dumps({
        base: {"bucketSize": 8, "threadsPerBlock": 128, "maxLevels": 30, "sample_ms": 2.0},
        base + "-l1": {"bucketSize": 16, "threadsPerBlock": 128, "maxLevels": 30, "sample_ms": 2.0},
        base + "-s1-l1": {"bucketSize": 24, "threadsPerBlock": 64, "maxLevels": 30, "sample_ms": 2.0}}))
    A._cache.clear()
    got = A.tune(clouds, queries, 32, dim=8, cache_path=str(path), lanes=(1,), max_queries_per_cloud=5)
    assert got["cached"] and got["key"] == base + "-l1" and got["bucketSize"] == 16
    got = A.tune(clouds, queries, 32, dim=8, cache_path=str(path), split_rules=(1,), lanes=(1,))
    assert got["key"] == base + "-s1-l1" and got["bucketSize"] == 24
    got = A.tune(clouds, queries, 32, dim=8, cache_path=str(path))
    assert got["key"] == base and got["bucketSize"] == 8
    A._cache.clear()
