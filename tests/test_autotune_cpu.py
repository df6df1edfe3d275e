"""Host logic of the batch autotuner (minirender_gb300/autotune.py) with a
fake context: every candidate timed, shapes that do not fit skipped, the
small_max stage run on the best shape, the winner applied and cached, the
cache reused by key."""
import json
from types import SimpleNamespace

import pytest

from minirender_gb300 import autotune as A
from minirender_gb300 import capi


class FakeCtx:
    """Times a candidate by a made-up cost; tile shapes wider than 64 do not
    fit (the library would refuse them), small_max 16 is the fastest."""

    def __init__(self):
        self.tiling = None
        self.small_max = None
        self.renders = 0
        self.applied = []

    def set_batch_tiling(self, tw, th, threads, chunk):
        if tw > 64:
            raise capi.MRError(-1, "tile does not fit")
        self.tiling = (tw, th, threads, chunk)
        self.applied.append(("tiling", self.tiling))

    def set_batch_small_max(self, v):
        self.small_max = v
        self.applied.append(("small_max", v))

    def set_batch_graphs(self, on):
        pass

    def set_profiling(self, on):
        pass

    def render_batch(self, *a):
        self.renders += 1

    def batch_stats(self):
        tw, th, threads, chunk = self.tiling
        ms = abs(tw * th - 1024) / 1024 + abs(threads - 128) / 256 + abs(chunk - 64) / 128 + 1.0
        ms += {0: 0.3, 16: 0.0, 64: 0.1, 256: 0.2}[self.small_max]
        return SimpleNamespace(stage_ms=[0.0, 0.0, 0.0, ms])


PREPARED = (None, 1, None, 1)


def test_tune_picks_fastest_and_caches(tmp_path):
    ctx = FakeCtx()
    path = str(tmp_path / "tune.json")
    best = A.tune(ctx, PREPARED, "k1", path=path)
    assert (best["tile_w"], best["tile_h"], best["threads"], best["chunk"]) == (32, 32, 128, 64)
    assert best["small_max"] == 16
    # every candidate that fits was timed, the refused ones skipped
    fits = [c for c in A.CANDIDATES if c[0] <= 64]
    timed = [r for r in best["table"] if r["small_max"] == A.DEFAULT_SMALL_MAX]
    assert len(timed) == len(fits)
    assert {r["small_max"] for r in best["table"]} == set(A.SMALL_MAX)
    # the winner is what the context was left with
    assert ctx.tiling == (32, 32, 128, 64) and ctx.small_max == 16
    with open(path) as f:
        assert json.load(f)["k1"]["small_max"] == 16


def test_cached_tuning_is_applied_without_timing(tmp_path):
    path = str(tmp_path / "tune.json")
    A.tune(FakeCtx(), PREPARED, "k1", path=path)
    ctx = FakeCtx()
    best = A.tune(ctx, PREPARED, "k1", path=path)
    assert ctx.renders == 0
    assert ctx.tiling == (best["tile_w"], best["tile_h"], best["threads"], best["chunk"])
    # another key is tuned afresh and both stay in the file
    ctx2 = FakeCtx()
    A.tune(ctx2, PREPARED, "k2", candidates=[(16, 16, 64, 32), (8, 8, 256, 128)], path=path)
    assert ctx2.renders > 0
    with open(path) as f:
        assert set(json.load(f)) == {"k1", "k2"}


def test_no_candidate_fits(tmp_path):
    with pytest.raises(RuntimeError):
        A.tune(FakeCtx(), PREPARED, "k", candidates=[(128, 8, 64, 32)], path=str(tmp_path / "t.json"))


def test_corrupt_cache_is_retuned(tmp_path):
    path = tmp_path / "tune.json"
    path.write_text("{ not json")
    best = A.tune(FakeCtx(), PREPARED, "k", candidates=[(16, 16, 64, 32)], path=str(path))
    assert json.loads(path.read_text())["k"]["tile_w"] == best["tile_w"] == 16


def test_batch_class_buckets():
    a = A.batch_class(256, 8_850_000, 256 * 640 * 480)
    b = A.batch_class(300, 9_000_000, 256 * 640 * 480)
    c = A.batch_class(8, 8_850_000, 256 * 640 * 480)
    assert a == b and a != c
