"""The batched form's worker autotuner: choice, cache and keys (no GPU; the
timing function is a stand-in)."""
import json

from contour3d_gb300 import autotune


def test_picks_the_fastest_and_caches_it(tmp_path):
    path = str(tmp_path / "tune.json")
    times = {2: 0.9, 4: 0.5, 6: 0.4, 8: 0.45, 12: 0.6}
    calls = []

    def run(w):
        calls.append(w)
        return times[w]

    first = autotune.tune("gpu|c20-p20-n64", run, path=path)
    assert first["workers"] == 6 and not first["cached"]
    assert sorted(calls) == sorted(times)
    second = autotune.tune("gpu|c20-p20-n64", run, path=path)
    assert second["workers"] == 6 and second["cached"]
    assert len(calls) == len(times)  # nothing measured again
    assert json.load(open(path))["gpu|c20-p20-n64"]["workers"] == 6


def test_keys_are_tuned_separately(tmp_path):
    path = str(tmp_path / "tune.json")
    a = autotune.tune("gpu|small", lambda w: {2: 1.0, 4: 2.0}[w], candidates=(2, 4), path=path)
    b = autotune.tune("gpu|large", lambda w: {2: 2.0, 4: 1.0}[w], candidates=(2, 4), path=path)
    assert (a["workers"], b["workers"]) == (2, 4)
    data = json.load(open(path))
    assert set(data) == {"gpu|small", "gpu|large"}


def test_unreadable_cache_is_replaced(tmp_path):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    r = autotune.tune("k", lambda w: float(w), candidates=(3, 1, 2), path=str(path))
    assert r["workers"] == 1 and not r["cached"]
    assert json.load(open(path))["k"]["workers"] == 1


def test_size_class():
    assert autotune.size_class([], []) == "empty"
    k = autotune.size_class([1 << 20] * 10, [1 << 20] * 10)
    assert k == "c20-p20-n8"
    assert autotune.size_class([1 << 24] * 64, [1 << 20] * 64) != k


def test_launch_shape_is_tuned_and_cached(tmp_path):
    path = str(tmp_path / "tune.json")
    calls = []

    def run(shape):
        calls.append(shape)
        return 1.0 if shape != (16, 8, 8) else 0.5

    r = autotune.tune_shape("gpu|shape|c20", run, path=path)
    assert r["shape"] == [16, 8, 8] and not r["cached"]
    assert len(calls) == len(autotune.SHAPES)
    r2 = autotune.tune_shape("gpu|shape|c20", run, path=path)
    assert r2["shape"] == [16, 8, 8] and r2["cached"] and len(calls) == len(autotune.SHAPES)


def test_tune_launch_shape_sets_the_choice(tmp_path):
    class FakeLib:
        def __init__(self):
            self.shape = None

        def set_launch_shape(self, *s):
            self.shape = s

    lib = FakeLib()
    r = autotune.tune_launch_shape(lib, lambda: None, [1 << 20], [1 << 20], "gpu", candidates=((32, 8, 8), (64, 4, 4)),
                                   repeats=1, path=str(tmp_path / "t.json"))
    assert lib.shape == tuple(r["shape"])
