"""Host logic of the launch autotuner (no GPU): choice, keys and the cache."""
import json

from xpbd_gpu import autotune


def test_pick_fastest_ignores_untimed():
    assert autotune.pick([3.0, None, 1.5, float("nan"), 1.5]) == 2
    assert autotune.pick([None, 2.0]) == 1


def test_pick_raises_without_timings():
    import pytest
    with pytest.raises(RuntimeError):
        autotune.pick([None, float("nan")])


def test_problem_key_is_order_independent():
    a = autotune.problem_key("single", "GB300", "1-2", tets=10, verts=5, block=1)
    b = autotune.problem_key("single", "GB300", "1-2", block=1, verts=5, tets=10)
    assert a == b and "tets=10" in a
    assert a != autotune.problem_key("single", "GB300", "1-3", tets=10, verts=5, block=1)


def test_cache_roundtrip(tmp_path):
    p = str(tmp_path / "sub" / "c.json")
    autotune._store_cache(p, "k1", {"scatter": "patch"})
    autotune._store_cache(p, "k2", {"scatter": "atomic"})
    data = json.load(open(p))
    assert data == {"k1": {"scatter": "patch"}, "k2": {"scatter": "atomic"}}
    assert autotune._load_cache(str(tmp_path / "missing.json")) == {}


def test_candidates_respect_per_tet_materials():
    all_c = autotune.single_candidates(per_tet_materials=False)
    assert {c[0] for c in all_c} == {"patch", "atomic", "gather"}
    assert {c[1] for c in all_c if c[0] == "patch"} == {64, 128, 256}
    per_tet = autotune.single_candidates(per_tet_materials=True)
    assert {c[0] for c in per_tet} == {"atomic", "gather"}


def test_cache_path_env(monkeypatch, tmp_path):
    monkeypatch.setenv("XPBD_AUTOTUNE_CACHE", str(tmp_path / "x.json"))
    assert autotune.cache_path() == str(tmp_path / "x.json")
