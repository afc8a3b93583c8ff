"""Host logic of the autotuner (no GPU): the result cache survives a JSON round trip through
BQA_GB300_TUNE_CACHE, a foreign or broken cache file is ignored, and plans describe
themselves with the variant names."""
import json

from bqa_gb300 import _lib, autotune


def test_cache_file_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("BQA_GB300_TUNE_CACHE", str(path))
    autotune.clear_cache()
    key = ("NVIDIA GB300", "single", 3, 16, 131072, True)
    autotune._CLASS_CACHE[key] = {"best": _lib.BQA_VARIANT_TILED, "ms": {1: 13.5, 2: 40.25}}
    jkey = ("NVIDIA GB300", "single", 16, ((3, 131072),))
    autotune._FORM_CACHE[jkey] = {"split": True, "ms": {"split": 13.9, "whole": 25.0}}
    autotune._save()
    autotune.clear_cache()
    monkeypatch.setattr(autotune, "_LOADED", False)
    autotune._load()
    assert autotune._CLASS_CACHE[key] == {"best": 1, "ms": {1: 13.5, 2: 40.25}}
    assert autotune._FORM_CACHE[jkey]["split"] is True
    autotune.clear_cache()


def test_broken_cache_file_is_ignored(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    monkeypatch.setenv("BQA_GB300_TUNE_CACHE", str(path))
    monkeypatch.setattr(autotune, "_LOADED", False)
    autotune.clear_cache()
    autotune._load()
    assert autotune._CLASS_CACHE == {}
    path.write_text(json.dumps({"classes": [[1, 2]]}))
    monkeypatch.setattr(autotune, "_LOADED", False)
    autotune._load()


def test_plan_description_and_buckets():
    p = autotune.Plan(chis=8, split=False, variants=[0, 1, 2], class_ms=[{}, {1: 0.5}, {2: 1.0}],
                      form_ms={"split": 2.0, "whole": 1.5})
    d = p.describe()
    assert d["form"] == "one-stage" and d["variants"] == ["default", "tiled", "generic"]
    assert d["class_ms"][1] == {"tiled": 0.5}
    assert [autotune._bucket(n) for n in (1, 2, 3, 1000, 1024, 1025)] == [1, 2, 4, 1024, 1024, 2048]



def test_only_missing_variants_are_skipped():
    """A candidate the library reports as unsupported is skipped; any other failure propagates."""
    assert autotune._missing_variant(_lib.BqaError("no tiled kernel", status=_lib.BQA_ERR_UNSUPPORTED))
    assert not autotune._missing_variant(_lib.BqaError("launch failed", status=3))
    assert not autotune._missing_variant(_lib.BqaError("bad argument", status=1))
