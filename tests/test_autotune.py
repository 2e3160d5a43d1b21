"""Autotuner bookkeeping on the CPU: size classes, cache keys, cache file round trip."""
import autotune


class FakeCtx:
    def __init__(self):
        self.calls = []

    def set_layout(self, layout):
        self.calls.append(("layout", layout))

    def set_batch_slots(self, slots):
        self.calls.append(("slots", slots))


def test_size_class_and_key():
    assert autotune.size_class(1) == 0 and autotune.size_class(1024) == 10 and autotune.size_class(1500) == 10
    assert autotune.size_class(0) == 0
    k1 = autotune.cache_key("GB300", 86, 1, 1, 1 << 20)
    assert k1 != autotune.cache_key("GB300", 86, 1, 2, 1 << 20)
    assert k1 == autotune.cache_key("GB300", 86, 1, 1, (1 << 20) + 5)


def test_cache_round_trip_and_apply(tmp_path):
    path = str(tmp_path / "cache.json")
    assert autotune.load_cache(path) == {}
    c = {"k": {"layout": "batched", "slots": 8}}
    autotune.store_cache(c, path)
    assert autotune.load_cache(path) == c
    ctx = FakeCtx()
    autotune.apply(ctx, c["k"])
    assert ctx.calls == [("layout", "batched"), ("slots", 8)]
    assert all(l in ("batched", "warp") and 1 <= s <= 32 for l, s in autotune.CANDIDATES)
