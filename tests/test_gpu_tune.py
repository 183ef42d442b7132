"""Autotuner of the fused slope + D8: every kernel variant it searches gives
the same bytes (and the oracle's D8), and its choice is persisted in the JSON
cache that a fresh context reads."""
import json
import math

import numpy as np
import pytest

from conftest import bits_equal
from gpu_helpers import d8_as_f64, dev, empty_dev, host, slope_close
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu

ND = -9999.0


def test_every_variant_gives_identical_bytes(ctx, oracle_lib, monkeypatch):
    dem = synth.hydro_dem(1003, 1301, seed=77, blob_fraction=0.08)   # nodata, ragged strips and segments
    d = dev(dem, 16)
    names = abi.focal_variant_names()
    assert len(names) >= 10 and len(set(names)) == len(names)
    outs = []
    for v in range(len(names)):
        monkeypatch.setenv("PARGO_FOCAL_VARIANT", str(v))
        assert ctx.focal_variant(dem.size) == v
        s = empty_dev(dem.shape, np.float32, 16)
        c = empty_dev(dem.shape, np.int8, 16)
        ctx.slope_d8(abi.raster(d, ND, 30.0), abi.raster(s, ND), abi.raster(c, -128))
        outs.append((host(s), host(c)))
    monkeypatch.delenv("PARGO_FOCAL_VARIANT")
    for v in range(1, len(names)):
        assert bits_equal(outs[v][0], outs[0][0]), names[v]
        assert np.array_equal(outs[v][1], outs[0][1]), names[v]
    assert bits_equal(d8_as_f64(outs[0][1], -128), oracle_lib.d8(dem, ND))
    ok, mx, _ = slope_close(outs[0][0], oracle_lib.slope(dem, ND, 30.0))
    assert ok, mx


def test_tuned_choice_persists_for_a_fresh_context(tmp_path, monkeypatch):
    cache = tmp_path / "sub" / "tune.json"
    monkeypatch.setenv("PARGO_TUNE_CACHE", str(cache))
    monkeypatch.delenv("PARGO_FOCAL_VARIANT", raising=False)
    dem = synth.slope_dem(2048, 2048, seed=5)
    cells = dem.size
    c1 = abi.Context(0)
    assert c1.focal_variant(cells) == 0                 # untuned, no cache: the size default
    d = dev(dem, 16)
    best, times = c1.tune_focal(abi.raster(d, ND, 30.0), reps=2)
    assert len(times) == len(abi.focal_variant_names()) and min(times) > 0
    assert times[best] == min(times)
    assert c1.focal_variant(cells) == best
    data = json.loads(cache.read_text())
    ent = [e for e in data["entries"] if e["op"] == "slope_d8"]
    assert len(ent) == 1
    assert ent[0]["size_class"] == int(math.log2(cells))
    assert ent[0]["variant"] == abi.focal_variant_names()[best]
    c1.close()
    c2 = abi.Context(0)                                 # a fresh context reads the cache
    assert c2.focal_variant(cells) == best
    assert c2.focal_variant(cells * 4) == abi.focal_variant_names().index("strip-s6x8-b5")  # other class: default
    c2.close()
    # a second tune of the same class replaces the entry; unknown names and junk are ignored
    data["entries"].append({"op": "slope_d8", "device": ent[0]["device"], "size_class": 10, "variant": "no-such"})
    cache.write_text(json.dumps(data))
    c3 = abi.Context(0)
    assert c3.focal_variant(1 << 10) == 0
    c3.tune_focal(abi.raster(d, ND, 30.0), reps=1)
    assert sum(1 for e in json.loads(cache.read_text())["entries"] if e["size_class"] == ent[0]["size_class"]) == 1
    c3.close()
    cache.write_text("{not json")
    c4 = abi.Context(0)
    assert c4.focal_variant(cells) == 0
    c4.close()
