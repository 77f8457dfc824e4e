"""Batched frames (hg_batch_*): many grooms with their own camera views and
deep opacity maps, one launch per pass, replayed as a CUDA graph.

Per item the batch must produce what the per-groom path (hg_groom_frame)
produces: the visibility G-buffers and deep opacity map bit for bit, colour
within float rounding; and one item is checked against the oracle frame.
"""
import numpy as np
import pytest

import oracle
from bevy_hair_gb300 import abi, configs
from bevy_hair_gb300.pipeline import HairBatch, HairRenderer

pytestmark = pytest.mark.gpu

VIS = (abi.BUF_CENTER, abi.BUF_CONSERVATIVE, abi.BUF_BETA, abi.BUF_DOM)
COLOUR = (abi.BUF_SHADED, abi.BUF_SHADED_DEPTH, abi.BUF_FILTERED, abi.BUF_FILTERED_DEPTH, abi.BUF_COLOR,
          abi.BUF_DEPTH)


@pytest.fixture(scope="module")
def renderer():
    r = HairRenderer(0)
    yield r
    r.close()


@pytest.fixture(scope="module")
def batch_scene():
    return configs.config4(scale=0.03, items=10)


def _make(renderer, bs):
    grooms = [renderer.upload(s.mesh) for s in bs.scenes]
    b = HairBatch(renderer, grooms, bs.sizes())
    params = [s.params() for s in bs.scenes]
    for k, (cam, dom) in enumerate(params):
        b.set_params(k, cam, dom)
    return b, grooms, params


def _read_all(b, n):
    return [{w: b.read(k, w) for w in VIS + COLOUR} for k in range(n)]


def _close(b, grooms):
    b.close()
    for g in grooms:
        g.close()


def _compare(got, want, colour_exact=False):
    for k, (g, w) in enumerate(zip(got, want)):
        for which in VIS:
            np.testing.assert_array_equal(g[which], w[which], err_msg=f"item {k} buffer {which}")
        for which in COLOUR:
            if colour_exact:
                np.testing.assert_array_equal(g[which], w[which], err_msg=f"item {k} buffer {which}")
            else:
                np.testing.assert_allclose(g[which], w[which], rtol=1e-5, atol=1e-6,
                                           err_msg=f"item {k} buffer {which}")


def test_batched_graph_frame_matches_per_groom_frames(renderer, batch_scene):
    bs = batch_scene
    lights = bs.light_array()
    b, grooms, _ = _make(renderer, bs)
    b.frame(lights, abi.BATCH_GRAPH)
    assert renderer.synchronize() == 0
    graph = _read_all(b, len(grooms))
    b.frame(lights, abi.BATCH_LAUNCHES)
    assert renderer.synchronize() == 0
    direct = _read_all(b, len(grooms))
    b.frame(lights, abi.BATCH_SEPARATE)
    assert renderer.synchronize() == 0
    separate = _read_all(b, len(grooms))
    _compare(graph, direct, colour_exact=True)
    _compare(graph, separate)
    # something was drawn in every item and every map
    for k, g in enumerate(graph):
        assert (g[abi.BUF_CENTER] != np.uint64(0xFFFFFFFFFFFFFFFF)).any(), k
    assert b.launches(abi.BATCH_GRAPH) <= 14
    assert b.launches(abi.BATCH_SEPARATE) == 18 * len(grooms)  # hg_groom_frame per item (camera raster: 3)
    _close(b, grooms)


def test_batched_item_visibility_matches_the_oracle(renderer, batch_scene):
    bs = batch_scene
    b, grooms, params = _make(renderer, bs)
    lights = bs.light_array()
    b.frame(lights)
    assert renderer.synchronize() == 0
    for k in (0, len(grooms) - 1):
        cam, dom = params[k]
        want = oracle.frame(bs.scenes[k].mesh, cam, dom, lights)
        np.testing.assert_array_equal(b.read(k, abi.BUF_CENTER), want["center"])
        np.testing.assert_array_equal(b.read(k, abi.BUF_CONSERVATIVE), want["cons"])
        np.testing.assert_array_equal(b.read(k, abi.BUF_BETA), want["beta"])
        np.testing.assert_array_equal(b.read(k, abi.BUF_DOM), want["dom"])
        np.testing.assert_allclose(b.read(k, abi.BUF_COLOR), want["color"], rtol=2e-3, atol=1e-5)
    _close(b, grooms)


def test_graph_replays_new_uniforms(renderer, batch_scene):
    bs = batch_scene
    b, grooms, params = _make(renderer, bs)
    lights = bs.light_array()
    b.frame(lights)
    renderer.synchronize()
    # move every camera: the graph uploads the new uniforms at replay
    for k, s in enumerate(bs.scenes):
        view = configs._camera(s.view.width, s.view.height, 800.0 + 20.0 * k, azimuth=0.4 * k)
        moved = configs.Scene(s.name, s.mesh, s.groom, view, s.dom_size, s.lights, s.directionals)
        cam, dom = moved.params()
        b.set_params(k, cam, dom)
    b.frame(lights, abi.BATCH_GRAPH)
    renderer.synchronize()
    graph = _read_all(b, len(grooms))
    b.frame(lights, abi.BATCH_SEPARATE)
    renderer.synchronize()
    _compare(graph, _read_all(b, len(grooms)))
    _close(b, grooms)


@pytest.mark.parametrize("mode", [abi.BATCH_GRAPH, abi.BATCH_LAUNCHES, abi.BATCH_SEPARATE])
def test_async_readback_lands_before_the_next_frame_composites(renderer, batch_scene, mode):
    """hg_batch_copy_out_async: every item's colour and depth copied on the
    copy stream while the next frame (moved cameras) is already enqueued; that
    frame waits for the copies before it writes the colour and depth targets."""
    torch = pytest.importorskip("torch")
    bs = batch_scene
    b, grooms, params = _make(renderer, bs)
    lights = bs.light_array()
    b.frame(lights, mode)
    renderer.synchronize()
    want = [(b.read(k, abi.BUF_COLOR).copy(), b.read(k, abi.BUF_DEPTH).copy()) for k in range(len(grooms))]
    b.frame(lights, mode)
    hosts = []
    for k, (c, d) in enumerate(want):
        hc = torch.empty(c.size, dtype=torch.float32, pin_memory=True)
        hd = torch.empty(d.size, dtype=torch.float32, pin_memory=True)
        assert renderer.lib.hg_batch_copy_out_async(b.handle, k, abi.BUF_COLOR, hc.data_ptr(), c.nbytes) == 0
        assert renderer.lib.hg_batch_copy_out_async(b.handle, k, abi.BUF_DEPTH, hd.data_ptr(), d.nbytes) == 0
        hosts.append((hc, hd))
    for k, s in enumerate(bs.scenes):
        view = configs._camera(s.view.width, s.view.height, 700.0 + 15.0 * k, azimuth=1.0 + 0.3 * k)
        moved = configs.Scene(s.name, s.mesh, s.groom, view, s.dom_size, s.lights, s.directionals)
        b.set_params(k, *moved.params())
    b.frame(lights, mode)
    renderer.copy_wait()
    assert renderer.synchronize() == 0
    changed = 0
    for k, ((c, d), (hc, hd)) in enumerate(zip(want, hosts)):
        np.testing.assert_array_equal(hc.numpy(), c, err_msg=f"item {k} colour")
        np.testing.assert_array_equal(hd.numpy(), d, err_msg=f"item {k} depth")
        changed += int(np.abs(b.read(k, abi.BUF_COLOR) - c).max() > 1e-3)
    assert changed >= len(grooms) // 2  # the moved frame did overwrite the targets
    _close(b, grooms)


def test_autotuner_picks_a_measured_shape(renderer, batch_scene):
    bs = batch_scene
    b, grooms, _ = _make(renderer, bs)
    lights = bs.light_array()
    results = b.tune(lights)
    assert len(results) >= 8 and all(r["ms"] > 0 for r in results)
    best = min(results, key=lambda r: r["ms"])
    chosen = b.tuning()
    assert {k: chosen[k] for k in ("raster_chunk", "tile_w", "filter_tile")} == \
           {k: best[k] for k in ("raster_chunk", "tile_w", "filter_tile")}
    b.frame(lights)
    renderer.synchronize()
    tuned = _read_all(b, len(grooms))
    b.frame(lights, abi.BATCH_SEPARATE)
    renderer.synchronize()
    _compare(tuned, _read_all(b, len(grooms)))
    _close(b, grooms)


@pytest.mark.parametrize("tile", [(16, 16, 1), (64, 4, 0)])
def test_every_tile_shape_gives_the_same_frame(renderer, batch_scene, tile):
    bs = batch_scene
    b, grooms, _ = _make(renderer, bs)
    lights = bs.light_array()
    b.frame(lights)
    renderer.synchronize()
    base = _read_all(b, len(grooms))
    b.set_tuning(tile_w=tile[0], tile_h=tile[1], filter_tile=tile[2], raster_chunk=1)
    b.frame(lights)
    renderer.synchronize()
    _compare(_read_all(b, len(grooms)), base)
    _close(b, grooms)


def test_batch_argument_errors(renderer, batch_scene):
    bs = batch_scene
    g0 = renderer.upload(bs.scenes[0].mesh)
    with pytest.raises(abi.HairGbError):
        HairBatch(renderer, [g0, g0], [bs.sizes()[0]] * 2)  # one groom twice
    b = HairBatch(renderer, [g0], [bs.sizes()[0]])
    with pytest.raises(abi.HairGbError):
        b.frame(bs.light_array())  # params not set
    cam, dom = bs.scenes[0].params()
    wrong = cam.copy()
    wrong["screen"][0] += 1
    with pytest.raises(abi.HairGbError):
        b.set_params(0, wrong, dom)
    with pytest.raises(abi.HairGbError):
        b.set_params(0, cam, None)  # the item has a map
    with pytest.raises(abi.HairGbError):
        b.set_tuning(tile_w=48)
    b.set_params(0, cam, dom)
    b.frame(bs.light_array())
    assert renderer.synchronize() == 0
    b.close()
    g0.close()


def test_full_size_batch_items_match_the_oracle(renderer):
    """The config 4 benchmark batch itself (64 grooms, 128 views) as one graph
    replay: three items (first, largest, last) against the oracle's frames."""
    bs = configs.config4(scale=1.0)
    b, grooms, params = _make(renderer, bs)
    lights = bs.light_array()
    b.frame(lights, abi.BATCH_GRAPH)
    assert renderer.synchronize() == 0
    largest = max(range(len(grooms)), key=lambda k: bs.scenes[k].mesh.strand_count())
    for k in sorted({0, largest, len(grooms) - 1}):
        cam, dom = params[k]
        want = oracle.frame(bs.scenes[k].mesh, cam, dom, lights)
        np.testing.assert_array_equal(b.read(k, abi.BUF_CENTER), want["center"])
        np.testing.assert_array_equal(b.read(k, abi.BUF_CONSERVATIVE), want["cons"])
        np.testing.assert_array_equal(b.read(k, abi.BUF_BETA), want["beta"])
        np.testing.assert_array_equal(b.read(k, abi.BUF_DOM), want["dom"])
        np.testing.assert_allclose(b.read(k, abi.BUF_COLOR), want["color"], rtol=2e-3, atol=1e-5)
    _close(b, grooms)


def test_graph_follows_a_new_light_probe(renderer, batch_scene):
    """hg_env_set after a graph was captured: the next graph frame must shade
    with the new probe (the captured graph held the old cubemaps' addresses),
    exactly as direct launches of the same frame do; and again after the probe
    is dropped."""
    from bevy_hair_gb300 import envmap

    bs = batch_scene
    b, grooms, _ = _make(renderer, bs)
    lights = bs.light_array()
    b.frame(lights, abi.BATCH_GRAPH)  # captured without a probe
    renderer.synchronize()
    no_probe = _read_all(b, len(grooms))
    for env in (envmap.procedural(size=64, levels=7, diffuse_size=8),
                envmap.procedural(seed=7, size=32, levels=6, diffuse_size=8), None):
        renderer.set_environment(env)
        b.frame(lights, abi.BATCH_GRAPH)
        assert renderer.synchronize() == 0
        graph = _read_all(b, len(grooms))
        b.frame(lights, abi.BATCH_LAUNCHES)
        assert renderer.synchronize() == 0
        _compare(graph, _read_all(b, len(grooms)), colour_exact=True)
        if env is not None:  # the probe lights the hair: colour changed
            assert any(np.abs(g[abi.BUF_SHADED] - w[abi.BUF_SHADED]).max() > 1e-4
                       for g, w in zip(graph, no_probe))
    _compare(graph, no_probe, colour_exact=True)
    _close(b, grooms)


def test_batched_frame_keeps_the_strand_cache_honest(renderer):
    """A batched frame rewrites each item's strand cache with the item's own
    transform.  A per-groom raster afterwards, with the transform the cache
    held before, must draw its own geometry (the cache is regenerated or
    ignored), not the batch's."""
    bs = configs.config4(scale=0.03, items=2)
    b, grooms, params = _make(renderer, bs)
    lights = bs.light_array()
    sc = bs.scenes[0]
    cam, dom = params[0]
    moved_cam, moved_dom = cam.copy(), dom.copy()
    for p in (moved_cam, moved_dom):
        p["world_from_model"][12] += 40.0  # translate the groom along x
    w, h, dw, dh = bs.sizes()[0]
    renderer.ensure_targets(w, h, dw, dh)
    g = grooms[0]
    renderer.generate(g, cam)  # cache at the original transform
    b.set_params(0, moved_cam, moved_dom)
    b.frame(lights, abi.BATCH_GRAPH)  # cache now at the moved transform
    assert renderer.synchronize() == 0
    renderer.clear_dom()
    renderer.lod(g, dom, abi.SLOT_DOM)
    renderer.scan(g, dom, abi.SLOT_DOM)
    renderer.raster(g, dom, abi.SLOT_DOM)  # every DOM strand is at 65 control points
    renderer.clear()
    renderer.lod(g, cam, abi.SLOT_CAMERA)
    renderer.scan(g, cam, abi.SLOT_CAMERA)
    renderer.raster(g, cam, abi.SLOT_CAMERA)
    assert renderer.synchronize() == 0
    cap = max(sc.mesh.strand_count(), 1)
    center, cons, beta = oracle.clear_targets(w, h)
    refs, total = oracle.scan(cam, oracle.lod(cam, sc.mesh), cap)
    oracle.raster(cam, sc.mesh, refs, total, center, cons, beta, None)
    d = oracle.clear_dom(dw, dh)
    drefs, dtotal = oracle.scan(dom, oracle.lod(dom, sc.mesh), cap)
    oracle.raster(dom, sc.mesh, drefs, dtotal, center, cons, beta, d)
    np.testing.assert_array_equal(renderer.read(abi.BUF_DOM)[:dw * dh], d[:dw * dh])
    np.testing.assert_array_equal(renderer.read(abi.BUF_CENTER), center)
    np.testing.assert_array_equal(renderer.read(abi.BUF_CONSERVATIVE), cons)
    _close(b, grooms)
