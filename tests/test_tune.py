"""The launch-shape autotuner (lmff_gb300/tune.py) on a GPU: it times every candidate on
graph-replayed NVE steps, returns the lowest-scoring one and caches it per (GPU,
precision, size bucket, element count); forces do not depend on the shape it picks."""
import json

import numpy as np
import pytest
from conftest import ILP, TERSOFF, rel_max

from lmff_gb300 import capi, structures, tune

pytestmark = pytest.mark.gpu


def test_tune_picks_lowest_score_and_caches(tmp_path, monkeypatch):
    monkeypatch.setattr(tune, "CACHE", str(tmp_path / "tune.json"))
    s = structures.thermalize(structures.ab_bilayer_graphene(8, 8), 300.0, seed=1)
    out = tune.tune(s, TERSOFF, ILP, elements=("C",), precision=capi.MIXED, tpas=(8, 32), blocks=(128,),
                    skins=(1.0,), tiles=(2, 1))
    cands = out["candidates"]
    assert len(cands) == 4 and not out["cached"]
    assert out["steps"] == 200   # ~2 M atom-steps for 512 atoms, capped at 200
    best = min(cands, key=lambda r: r["score_ms"])
    assert (out["tpa"], out["block"], out["skin"], out["tile"]) == (best["tpa"], best["block"], best["skin"],
                                                                     best["tile"])
    assert all(r["step_ms"] > 0 for r in cands)
    again = tune.tune(s, TERSOFF, ILP, elements=("C",), precision=capi.MIXED, tpas=(8, 32), blocks=(128,),
                      skins=(1.0,), tiles=(2, 1))
    assert again["cached"] and again["tpa"] == out["tpa"]
    assert out["key"] in json.load(open(tmp_path / "tune.json"))


def test_forces_independent_of_launch_shape():
    s = structures.thermalize(structures.ab_bilayer_graphene(8, 8), 300.0, seed=1)
    ref = None
    for tpa, block, tile in [(8, 128, 2), (16, 64, 1), (32, 256, 2), (4, 128, 1)]:
        eng = capi.Engine(TERSOFF, ILP, elements=("C",), precision=capi.MIXED, skin=1.0)
        eng.set_option("tpa", tpa)
        eng.set_option("block", block)
        eng.set_option("pair_tile", tile)
        f = eng.compute_system(s)["f"]
        eng.close()
        if ref is None:
            ref = f
        else:
            assert rel_max(f, ref) <= 1e-6, (tpa, block, tile)
    assert np.isfinite(ref).all()
