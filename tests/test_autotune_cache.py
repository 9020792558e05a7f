"""The autotuner's choice cache (host only, no device work): classes by total and mean world cells,
nearest-class fallback on the same device, and argument checks."""
from __future__ import annotations

import pytest

import master_thesis_gb300 as T


@pytest.fixture(autouse=True)
def clean_cache():
    T.autotune_clear()
    yield
    T.autotune_clear()


def test_empty_cache_finds_nothing():
    assert T.autotune_lookup(0, 1 << 20, 4) is None


def test_record_and_exact_lookup():
    T.autotune_record(0, 48_000_000, 256, 3, 9, 2)
    assert T.autotune_lookup(0, 48_000_000, 256) == (3, 9, 2)
    # same half-octave classes
    assert T.autotune_lookup(0, 49_000_000, 256) == (3, 9, 2)


def test_nearest_class_on_the_same_device():
    T.autotune_record(0, 1 << 16, 1, 1, 8, 1)      # small single world
    T.autotune_record(0, 1 << 26, 256, 4, 11, 4)   # large batch
    assert T.autotune_lookup(0, 1 << 17, 1) == (1, 8, 1)
    assert T.autotune_lookup(0, 1 << 25, 200) == (4, 11, 4)
    assert T.autotune_lookup(1, 1 << 26, 256) is None  # other device: nothing tuned


def test_later_record_replaces():
    T.autotune_record(0, 1 << 22, 1, 2, 8, 1)
    T.autotune_record(0, 1 << 22, 1, 5, 10, 3)
    assert T.autotune_lookup(0, 1 << 22, 1) == (5, 10, 3)


@pytest.mark.parametrize("args", [(0, 1 << 20, 1, 0, 8, 1), (0, 1 << 20, 1, 10, 8, 1), (0, 1 << 20, 1, 4, 7, 1),
                                  (0, 1 << 20, 1, 4, 12, 1), (0, 0, 1, 4, 8, 1), (0, 1 << 20, 0, 4, 8, 1),
                                  (-1, 1 << 20, 1, 4, 8, 1), (0, 1 << 20, 1, 4, 8, 0), (0, 1 << 20, 1, 4, 8, 6)])
def test_invalid_records_rejected(args):
    with pytest.raises(T.TectoError):
        T.autotune_record(*args)
