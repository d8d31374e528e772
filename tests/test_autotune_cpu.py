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
