"""The batched-QR autotuner's cache key (host logic, no GPU): batches with the same size mix share
a tuning result, different mixes or devices do not."""
from later_gb300 import autotune


def test_same_mix_same_key():
    a = [(1000, 64), (5000, 200), (300, 20)] * 10
    b = list(reversed(a))  # order does not matter
    assert autotune._key(a, "GB300") == autotune._key(b, "GB300")


def test_scaled_batch_same_key():
    # the key is a normalised histogram: twice the batch with the same mix shares the result
    a = [(1000, 64), (5000, 200)] * 8
    assert autotune._key(a, "GB300") == autotune._key(a * 2, "GB300")


def test_batch_count_bucket():
    # the same mix at 10 and at 10,000 matrices is tuned separately (factor-of-4 count buckets)
    a = [(1000, 64), (5000, 200)] * 5
    assert autotune._key(a, "GB300") != autotune._key(a * 1000, "GB300")


def test_different_mix_or_device_different_key():
    a = [(1000, 64)] * 10
    b = [(8000, 250)] * 10
    assert autotune._key(a, "GB300") != autotune._key(b, "GB300")
    assert autotune._key(a, "GB300") != autotune._key(a, "other")


def test_cache_path_override(tmp_path, monkeypatch):
    monkeypatch.setenv("LATER_GB300_TUNE_CACHE", str(tmp_path / "t.json"))
    assert autotune._cache_path() == tmp_path / "t.json"
