"""The launch-shape autotuner: cache file, keys and selection on the CPU;
on the GPU, that every candidate launch shape gives identical results and
that a tuned tree uses its cached shape."""

import json

import numpy as np
import pytest

from numba_celltree_gb300 import autotune as at
from numba_celltree_gb300 import synthetic as syn


def test_buckets_and_keys():
    assert [at.bucket(n) for n in (0, 1, 2, 3, 5, 1000, 1 << 20, 3 << 20)] == [0, 0, 1, 2, 2, 10, 20, 22]
    k1 = at.cache_key("locate", "GPU|sm152|cc10.3", 16_000_000, 268_435_456, K=3)
    k2 = at.cache_key("locate", "GPU|sm152|cc10.3", 17_000_000, 250_000_000, K=3)
    k3 = at.cache_key("locate", "GPU|sm152|cc10.3", 16_000_000, 268_435_456, K=4)
    assert k1 == k2 != k3
    assert k1 == "locate|GPU|sm152|cc10.3|c24|q28|K3"


def test_candidates_cover_the_space():
    c = at.candidates("locate")
    assert len(c) == 4 * 3 * 3 and len({json.dumps(x, sort_keys=True) for x in c}) == len(c)
    c = at.candidates("boxes", fixed={"work_order": True})
    assert len(c) == 3 and all(x["work_order"] is True for x in c)


def test_pick_and_cache_round_trip(tmp_path, monkeypatch):
    assert at.pick([({"a": 1}, 3.0), ({"a": 2}, 2.0), ({"a": 3}, 2.0)]) == ({"a": 2}, 2.0)
    with pytest.raises(ValueError):
        at.pick([])
    path = tmp_path / "t.json"
    monkeypatch.setenv(at.CACHE_ENV, str(path))
    c = at.cache()
    assert c.path == path and c.get("x") is None
    c.put("x", {"config": {"threads": 128, "work_order": False}, "ms": 1.0})
    d = json.loads(path.read_text())
    assert d["format"] == 1 and d["entries"]["x"]["config"]["threads"] == 128
    # another process's entry is merged, not lost
    d["entries"]["y"] = {"config": {"threads": 64}}
    path.write_text(json.dumps(d))
    at.TuningCache(path).put("z", {"config": {}})
    assert set(json.loads(path.read_text())["entries"]) == {"x", "y", "z"}
    # lookup merges over the defaults and ignores unknown knobs
    at._cache = None
    cfg = at.lookup("boxes", "x")
    assert cfg == dict(at.DEFAULTS["boxes"], threads=128, work_order=False)
    assert at.lookup("boxes", "missing") == at.DEFAULTS["boxes"]
    # a damaged file reads as empty and is rewritten on the next put
    path.write_text("{not json")
    assert at.TuningCache(path).get("x") is None
    at.TuningCache(path).put("w", {"config": {}})
    assert "w" in json.loads(path.read_text())["entries"]
    monkeypatch.setenv(at.MODE_ENV, "0")
    assert not at.enabled()
    monkeypatch.setenv(at.MODE_ENV, "1")
    assert at.enabled()


def test_tune_selects_the_fastest_with_a_fake_clock(tmp_path, monkeypatch):
    monkeypatch.setenv(at.CACHE_ENV, str(tmp_path / "t.json"))
    at._cache = None
    cost = {64: 3.0, 128: 1.0, 256: 2.0}
    monkeypatch.setattr(at, "time_gpu", lambda fn, reps=3: (fn(), cost[seen[-1]])[1])
    seen = []
    e = at.tune("boxes", "k", lambda c: seen.append(c["threads"]), at.candidates("boxes", {"work_order": None}),
                default={"threads": 256, "work_order": None})
    assert e["config"]["threads"] == 128 and e["ms"] == 1.0 and e["default_ms"] == 2.0
    assert at.cache().get("k")["config"]["threads"] == 128


@pytest.mark.gpu
def test_every_launch_shape_gives_identical_results():
    import torch

    from numba_celltree_gb300 import CellTree2d

    xy, f = syn.triangle_mesh(200, seed=91, extent=(200.0, 200.0), offset=(5.0e5, 4.2e6))
    tree = CellTree2d(xy, f, -1)
    t = tree._tree
    pts = syn.uniform_points(300_000, xy.min(0), xy.max(0), seed=92, margin=0.01)
    pts[::100] = syn.near_edge_points(xy, f, len(pts[::100]), dist=1e-9, seed=93)
    p_d = torch.as_tensor(pts, device="cuda")
    tol = tree.default_tolerance()
    ref = torch.empty(len(pts), dtype=torch.int64, device="cuda")
    t.locate(p_d, ref, tol, "fp64", config={"stack": 0})
    out = torch.empty_like(ref)
    for cfg in at.candidates("locate"):
        out.fill_(-7)
        t.locate(p_d, out, tol, "fp32", config=cfg)
        assert torch.equal(out, ref), cfg
    for cfg in at.candidates("fp64"):
        t.locate(p_d, out, tol, "fp64", config=cfg)
        assert torch.equal(out, ref), cfg
    boxes = torch.as_tensor(syn.random_boxes(80_000, xy.min(0), xy.max(0), 0.1, 8.0, seed=94, log_uniform=True),
                            device="cuda")
    base = t.locate_boxes(boxes, dict(at.DEFAULTS["boxes"]))
    for cfg in at.candidates("boxes"):
        got = t.locate_boxes(boxes, cfg)
        assert all(torch.equal(a, b) for a, b in zip(got, base)), cfg
    rng = np.random.default_rng(95)
    a0 = rng.uniform(xy.min(0), xy.max(0), (70_000, 2))
    segs = torch.as_tensor(np.stack([a0, a0 + rng.uniform(-5, 5, (70_000, 2))], 1), device="cuda")
    base = t.locate_edges(segs, 1, dict(at.DEFAULTS["segments"]))
    for cfg in at.candidates("segments"):
        got = t.locate_edges(segs, 1, cfg)
        assert all(torch.equal(a, b) for a, b in zip(got, base)), cfg
    for dens in at.SPACE["index"]["grid_density"]:
        t.rebuild_index(dens)
        t.locate(p_d, out, tol, "fp32")
        assert torch.equal(out, ref), dens


@pytest.mark.gpu
def test_first_use_tuning_is_cached_and_applied(tmp_path, monkeypatch):
    import torch

    from numba_celltree_gb300 import CellTree2d

    monkeypatch.setenv(at.CACHE_ENV, str(tmp_path / "tuning.json"))
    at._cache = None
    xy, f = syn.triangle_mesh(300, seed=96)
    tree = CellTree2d(xy, f, -1)
    pts = syn.uniform_points(1 << 20, (0, 0), (1, 1), seed=97)
    expected = tree.locate_points(pts[:1000])
    got = tree.locate_points(torch.as_tensor(pts, device="cuda"))  # tunes (first use), then locates
    assert np.array_equal(got[:1000].cpu().numpy(), expected)
    key = tree._tree.tune_key("locate", 1 << 20)
    entry = json.loads((tmp_path / "tuning.json").read_text())["entries"][key]
    assert entry["candidates"] >= 8 and entry["ms"] > 0
    assert tree._tree.cached("locate", 1 << 20)["cells_bpsm"] == entry["config"]["cells_bpsm"]
    # a fresh tree of the same size class reads the cache instead of tuning again
    tree2 = CellTree2d(xy, f, -1)
    assert tree2._tree.cached("locate", 1 << 20) == tree._tree.cached("locate", 1 << 20)
    # explicit tuning of the index density and of the box traversal
    res = tree.autotune(points=pts[:200_000], boxes=syn.random_boxes(70_000, (0, 0), (1, 1), 0.001, 0.02, seed=98),
                        index=True)
    assert set(res) == {"index", "locate", "boxes"}
    assert np.array_equal(tree.locate_points(pts[:1000]), expected)
