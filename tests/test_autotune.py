"""The autotuner's choice and cache on the CPU, with a stand-in timing function."""
from kazan_gb300 import autotune


def test_candidates():
    assert len(autotune.candidates(ordered=True)) == 8
    opaque = autotune.candidates(ordered=False)
    assert {c.tile for c in opaque} == {16}
    assert [c.mode for c in opaque[:2]] == ["batched", "persistent"]
    # each knob varied alone, in the batched schedule, the others at their defaults
    varied = opaque[2:]
    assert all(c.mode == "batched" for c in varied) and len(set(varied)) == len(varied)
    for c in varied:
        assert sum(getattr(c, k) != v for k, v in autotune.DEFAULTS.items()) == 1
    assert {c.warp_px for c in varied} >= set(autotune.WARP_PX)
    assert [c.label() for c in opaque[:3]] == ["batched/16", "persistent/16", "batched/16/warp_px96"]
    assert autotune.candidates(ordered=False, knobs=False) == opaque[:2]


def test_knob_choice_round_trips_through_the_cache(tmp_path):
    path = str(tmp_path / "tune.json")

    def timer(c):
        return 1.0 if (c.warp_px, c.geo_blocks) == (256, 0) else 2.0

    sig = autotune.signature("GB300", False, 4096, 32_650_790, 2048, 2048)
    best, table = autotune.Tuner(path).choose(sig, timer, autotune.candidates(ordered=False))
    assert (best.mode, best.warp_px, best.job_blocks) == ("batched", 256, 16) and table[best] == 1.0
    again, table2 = autotune.Tuner(path).choose(sig, timer, autotune.candidates(ordered=False))
    assert again == best and table2 is None
    assert best.options() == {"mode": "batched", "tile": 16, "warp_px": 256, "job_blocks": 16, "geo_blocks": 0}


def test_tune_picks_fastest_and_breaks_ties_towards_batched():
    times = {("batched", 16): 2.0, ("persistent", 16): 1.5, ("batched", 32): 1.5, ("persistent", 32): 3.0}
    best, table = autotune.tune(lambda c: times[(c.mode, c.tile)],
                                [autotune.Config(m, t) for (m, t) in times])
    assert (best.mode, best.tile) == ("batched", 32) and len(table) == 4


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "tune.json")
    calls = []

    def timer(c):
        calls.append(c)
        return {8: 3.0, 16: 1.0, 32: 2.0, 64: 4.0}[c.tile] + (0.5 if c.mode == "persistent" else 0.0)

    sig = autotune.signature("GB300", True, 4096, 32_650_790, 2048, 2048)
    best, table = autotune.Tuner(path).choose(sig, timer, autotune.candidates())
    assert (best.mode, best.tile) == ("batched", 16) and table is not None and len(calls) == 8
    again, table2 = autotune.Tuner(path).choose(sig, timer, autotune.candidates())
    assert again == best and table2 is None and len(calls) == 8
    other = autotune.signature("GB300", False, 4096, 32_650_790, 2048, 2048)
    assert autotune.Tuner(path).lookup(other) is None


def test_signature_buckets():
    a = autotune.signature("g", False, 4096, 32_000_000, 2048, 2048)
    b = autotune.signature("g", False, 4000, 33_000_000, 2048, 2048)
    c = autotune.signature("g", False, 64, 32_000_000, 2048, 2048)
    assert a == b != c
