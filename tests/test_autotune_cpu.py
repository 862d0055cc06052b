"""Autotuner host logic: cache keys, the JSON cache and the cached-choice path (a stand-in timer; the
device timing runs in the GPU tests)."""
import json

from voxhenry_gb300 import autotune


class FakeGeom:
    tuning = None


def test_keys_group_batch_widths_and_separate_shapes():
    k = autotune.tuning_key((512, 512, 16), (311, 10), "fp32", 16, device="GB300")
    assert k == autotune.tuning_key((512, 512, 16), (311, 10), "fp32", 9, device="GB300")    # 9..16 share
    assert k != autotune.tuning_key((512, 512, 16), (311, 10), "fp32", 17, device="GB300")
    assert k != autotune.tuning_key((512, 512, 16), (311, 10), "df", 16, device="GB300")
    assert k != autotune.tuning_key((256, 256, 8), (311, 10), "fp32", 16, device="GB300")
    # a rebuilt library (other kernel sources) does not reuse the choices timed on the old one
    assert autotune.tuning_key((512, 512, 16), (311, 10), "fp32", 16, device="GB300", lib="0123456789ab") != \
        autotune.tuning_key((512, 512, 16), (311, 10), "fp32", 16, device="GB300", lib="ba9876543210")
    assert "|lib=" in k


def test_tune_times_once_then_uses_the_cache(tmp_path):
    path = str(tmp_path / "t.json")
    calls = []

    def timer(geom, prec, B):
        calls.append((prec, B))
        return {"y_variant": 2, "z_variant": 1, "max_rhs": 8, "ms_per_rhs": 0.5}

    g = FakeGeom()
    a = autotune.tune(g, "fp32", 12, (64, 16, 16), (16, 16), path=path, timer=timer)
    assert a["cached"] is False and calls == [("fp32", 12)]
    b = autotune.tune(g, "fp32", 16, (64, 16, 16), (16, 16), path=path, timer=timer)   # same bucket
    assert b["cached"] is True and len(calls) == 1 and g.tuning == ("fp32", 2, 1, 8, 0)
    autotune.tune(g, "fp32", 12, (64, 16, 16), (16, 16), path=path, timer=timer, retune=True)
    assert len(calls) == 2
    d = json.load(open(path))
    assert len(d) == 1 and list(d.values())[0]["max_rhs"] == 8


def test_corrupt_cache_is_ignored(tmp_path):
    path = tmp_path / "t.json"
    path.write_text("not json")
    assert autotune.load_cache(str(path)) == {}
