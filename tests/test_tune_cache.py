"""The autotuner's cache file (rd_tune_cache_get / rd_tune_cache_put): a
round trip through the C ABI with no device involved - keys kept apart, the
last line of a key winning, malformed lines skipped, bad keys refused."""
import pytest


def test_cache_round_trip_without_a_device(pkg, tmp_path):
    pkg.build()
    path = str(tmp_path / "tune.txt")
    key_a = "sm103 sms152 fp32 lagged1 trackfp0 scenes1 particles1100000 nodes2097152 grid128x128x128"
    key_b = "sm103 sms152 fp32 lagged1 trackfp0 scenes64 particles3924026 nodes36706709 grid127x127x127"
    assert pkg.tune_cache_get(path, key_a) is None  # no file yet
    pkg.tune_cache_put(path, key_a, 256, 3, pkg.SCATTER_LANE_PAIRS, 0.2508)
    pkg.tune_cache_put(path, key_b, 192, 2, pkg.SCATTER_RECORD_PAIRS, 1.05)
    a = pkg.tune_cache_get(path, key_a)
    assert (a["particles_per_item"], a["ctas_per_sm"], a["scatter"], a["from_cache"]) == (256, 3, "lane_pairs", True)
    assert a["ms_per_step"] == pytest.approx(0.2508)
    b = pkg.tune_cache_get(path, key_b)
    assert (b["particles_per_item"], b["ctas_per_sm"], b["scatter"]) == (192, 2, "record_pairs")
    # a later line for the same key wins; garbage and a key that only shares a prefix are ignored
    with open(path, "a") as f:
        f.write("not a record\n" + key_a + "\tthree 2 1 0.1\n" + key_a + "x\t64 1 0 0.5\n")
    pkg.tune_cache_put(path, key_a, 128, 1, pkg.SCATTER_RECORD_PAIRS, 0.30)
    a = pkg.tune_cache_get(path, key_a)
    assert (a["particles_per_item"], a["ctas_per_sm"], a["scatter"]) == (128, 1, "record_pairs")
    assert pkg.tune_cache_get(path, "sm90 other") is None
    for bad in ("", "tab\tin key", "new\nline"):
        with pytest.raises(pkg.RDError):
            pkg.tune_cache_put(path, bad, 128, 1)
    with pytest.raises(pkg.RDError):
        pkg.tune_cache_put(path, key_a, 128, 1, 7)  # no such scatter layout
