"""Parity of the CUDA passes with the CPU oracle, through the C ABI.

Visibility outputs (LodRecords, StrandRefs, center / conservative / beta
G-buffers, deep opacity map) must be bit-exact.  Shaded colour is compared on
identical inputs (the GPU's own G-buffer and map fed to the oracle) within
SHADE_RTOL / SHADE_ATOL; the filter's coverage alpha is exact and its colour
within FILTER_RTOL.
"""
import math
import os
from pathlib import Path

import numpy as np
import pytest

import oracle
from bevy_hair_gb300 import abi, configs, host
from bevy_hair_gb300.pipeline import HairRenderer, Light, pack_lights

pytestmark = pytest.mark.gpu

# Colour tolerances: the GPU evaluates exp/log/asin/cos/pow with CUDA's
# functions and FMA contraction, the oracle with libm and none.
SHADE_RTOL, SHADE_ATOL = 2e-3, 1e-5
FILTER_RTOL, FILTER_ATOL = 1e-4, 1e-6
EMPTY = np.uint64(0xFFFFFFFFFFFFFFFF)


@pytest.fixture(scope="module")
def renderer():
    r = HairRenderer(0)
    yield r
    r.close()


def _assert_equal(name, got, want):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape, (name, got.shape, want.shape)
    bad = np.flatnonzero(got != want)
    if bad.size:
        i = bad[:5]
        pytest.fail(f"{name}: {bad.size} of {got.size} differ; first {i.tolist()}: got {got[i].tolist()} "
                    f"want {want[i].tolist()}")


def _scenes():
    return {
        "config1": lambda: configs.config1(scale=0.05),
        "config2": lambda: configs.config2(scale=0.02),
        "config3": lambda: configs.config3(scale=0.01),
    }


def _visibility(r: HairRenderer, sc: configs.Scene, cam, dom, scene_depth=None):
    w, h = int(cam["screen"][0]), int(cam["screen"][1])
    r.ensure_targets(w, h, *sc.dom_size)
    g = r.upload(sc.mesh)
    depth_ptr = None
    if scene_depth is not None:
        r.write(abi.BUF_DEPTH, scene_depth)
        depth_ptr, _ = r.buffer(abi.BUF_DEPTH)
    r.clear()
    r.lod(g, cam, abi.SLOT_CAMERA)
    r.scan(g, cam, abi.SLOT_CAMERA)
    r.raster(g, cam, abi.SLOT_CAMERA, depth_ptr)
    out = {"lod": g.read(abi.SLOT_CAMERA, abi.GBUF_LOD), "refs": g.read(abi.SLOT_CAMERA, abi.GBUF_REFS),
           "indirect": g.read(abi.SLOT_CAMERA, abi.GBUF_INDIRECT)}
    out["center"] = r.read(abi.BUF_CENTER)
    out["cons"] = r.read(abi.BUF_CONSERVATIVE)
    out["beta"] = r.read(abi.BUF_BETA)
    if dom is not None:
        r.clear_dom()
        r.lod(g, dom, abi.SLOT_DOM)
        r.scan(g, dom, abi.SLOT_DOM)
        r.raster(g, dom, abi.SLOT_DOM)
        out["dom_depth"] = r.read(abi.BUF_DOM)
        r.raster(g, host.dom_layers_params(dom), abi.SLOT_DOM)
        out["dom"] = r.read(abi.BUF_DOM)
        out["dom_lod"] = g.read(abi.SLOT_DOM, abi.GBUF_LOD)
        out["dom_refs"] = g.read(abi.SLOT_DOM, abi.GBUF_REFS)
        out["dom_indirect"] = g.read(abi.SLOT_DOM, abi.GBUF_INDIRECT)
    assert r.synchronize() == 0
    g.close()
    return out


def _oracle_visibility(sc, cam, dom, scene_depth=None):
    w, h = int(cam["screen"][0]), int(cam["screen"][1])
    cap = max(sc.mesh.strand_count(), 1)
    center, cons, beta = oracle.clear_targets(w, h)
    lod = oracle.lod(cam, sc.mesh)
    refs, total = oracle.scan(cam, lod, cap)
    counts = oracle.raster(cam, sc.mesh, refs, total, center, cons, beta, None, scene_depth)
    out = dict(lod=lod, refs=refs, total=total, center=center, cons=cons, beta=beta, counts=counts)
    if dom is not None:
        d = oracle.clear_dom(*sc.dom_size)
        dl = oracle.lod(dom, sc.mesh)
        drefs, dtotal = oracle.scan(dom, dl, cap)
        oracle.raster(dom, sc.mesh, drefs, dtotal, center, cons, beta, d)
        out["dom_depth"] = d.copy()
        oracle.raster(host.dom_layers_params(dom), sc.mesh, drefs, dtotal, center, cons, beta, d)
        out.update(dom=d, dom_lod=dl, dom_refs=drefs, dom_total=dtotal)
    return out


def _check_visibility(got, want, with_dom=True):
    n = len(want["lod"])
    _assert_equal("lod", got["lod"][:n].view(np.uint32), want["lod"].view(np.uint32))
    total = int(got["indirect"][0])
    assert total == want["total"]
    assert got["indirect"][1] == 1 and got["indirect"][2] == 1
    _assert_equal("refs", got["refs"][:total].view(np.uint32), want["refs"][:total].view(np.uint32))
    _assert_equal("center", got["center"], want["center"])
    _assert_equal("conservative", got["cons"], want["cons"])
    _assert_equal("beta", got["beta"], want["beta"])
    if with_dom:
        _assert_equal("dom_lod", got["dom_lod"][: len(want["dom_lod"])].view(np.uint32),
                      want["dom_lod"].view(np.uint32))
        assert int(got["dom_indirect"][0]) == want["dom_total"]
        _assert_equal("dom depth pass", got["dom_depth"], want["dom_depth"])
        _assert_equal("dom layers pass", got["dom"], want["dom"])


@pytest.mark.parametrize("name", list(_scenes()))
def test_visibility_and_dom_bit_exact(renderer, name):
    sc = _scenes()[name]()
    cam, dom = sc.params()
    got = _visibility(renderer, sc, cam, dom)
    want = _oracle_visibility(sc, cam, dom)
    assert (want["center"] != EMPTY).sum() > 100, "scene draws too little to be a test"
    _check_visibility(got, want)


@pytest.mark.parametrize("name", ["config2", "config3_far"])
def test_strand_cache_gives_the_same_visibility(renderer, name):
    """hg_generate then the rasters: refs at 65 control points read the strand
    cache, the others generate in the raster; the buffers must not change."""
    if name == "config2":
        sc = configs.config2(scale=0.02)
    else:  # LOD levels: only part of the camera refs are at 65 control points
        sc = configs.config3(scale=0.01)
        sc.view = configs._camera(sc.view.width, sc.view.height, 1200.0)
        sc.groom.lam = 1.0
    cam, dom = sc.params()
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.generate(g, cam)
    renderer.clear()
    renderer.lod(g, cam, abi.SLOT_CAMERA)
    renderer.scan(g, cam, abi.SLOT_CAMERA)
    renderer.raster(g, cam, abi.SLOT_CAMERA)
    renderer.clear_dom()
    renderer.lod(g, dom, abi.SLOT_DOM)
    renderer.scan(g, dom, abi.SLOT_DOM)
    renderer.raster(g, dom, abi.SLOT_DOM)
    renderer.raster(g, host.dom_layers_params(dom), abi.SLOT_DOM)
    assert renderer.synchronize() == 0
    want = _oracle_visibility(sc, cam, dom)
    _assert_equal("center", renderer.read(abi.BUF_CENTER), want["center"])
    _assert_equal("conservative", renderer.read(abi.BUF_CONSERVATIVE), want["cons"])
    _assert_equal("beta", renderer.read(abi.BUF_BETA), want["beta"])
    _assert_equal("dom", renderer.read(abi.BUF_DOM), want["dom"])
    cps = want["lod"]["control_points"][want["lod"]["n_lod"] > 0]
    if name != "config2":
        assert (cps == 65).any() and (cps != 65).any()
    g.close()


def test_dense_groom_with_tile_depth_rejection(renderer):
    """A dense groom at low resolution (deep overdraw) with a small deep
    opacity map: the later stages of the camera and DOM depth passes skip most
    segments behind the tile depths, and no buffer may change."""
    sc = configs.config2(scale=0.25)
    sc.view = configs._camera(384, 216, 900.0)
    sc.dom_size = (192, 192)
    cam, dom = sc.params()
    got = _visibility(renderer, sc, cam, dom)
    want = _oracle_visibility(sc, cam, dom)
    _check_visibility(got, want)
    covered = int((want["center"] != EMPTY).sum())
    assert covered > 5000 and want["counts"]["samples"] > 50 * covered


def test_two_grooms_into_one_g_buffer(renderer):
    """A second groom rastered over the first without a clear: the tile depths
    of its later stages start from the first groom's words."""
    a = configs.config2(scale=0.05)
    b = configs.config3(scale=0.02)
    a.view = configs._camera(480, 270, 900.0)
    cam_a, _ = a.params()
    b.view = a.view
    cam_b, _ = b.params()
    renderer.ensure_targets(480, 270, *a.dom_size)
    ga, gb = renderer.upload(a.mesh), renderer.upload(b.mesh)
    renderer.clear()
    for g, cam in ((ga, cam_a), (gb, cam_b)):
        renderer.lod(g, cam, abi.SLOT_CAMERA)
        renderer.scan(g, cam, abi.SLOT_CAMERA)
        renderer.raster(g, cam, abi.SLOT_CAMERA)
    assert renderer.synchronize() == 0
    center, cons, beta = oracle.clear_targets(480, 270)
    for sc, cam in ((a, cam_a), (b, cam_b)):
        lod = oracle.lod(cam, sc.mesh)
        refs, total = oracle.scan(cam, lod, max(sc.mesh.strand_count(), 1))
        oracle.raster(cam, sc.mesh, refs, total, center, cons, beta, None)
    _assert_equal("center", renderer.read(abi.BUF_CENTER), center)
    _assert_equal("conservative", renderer.read(abi.BUF_CONSERVATIVE), cons)
    _assert_equal("beta", renderer.read(abi.BUF_BETA), beta)
    assert (center != EMPTY).sum() > 1000
    ga.close()
    gb.close()


@pytest.mark.parametrize("diameter", [0.01, 0.3, 0.7, 1.0, 1.41421356, 2.5])
def test_center_disk_diameters(renderer, diameter):
    """The centre-sample acceptance disk (raster.wgsl:201,212) at several
    diameters, including the 0.05 floor and one whose radius squares inexactly."""
    sc = configs.config1(scale=0.03)
    sc.groom.center_diameter = diameter
    cam, dom = sc.params()
    got = _visibility(renderer, sc, cam, None)
    want = _oracle_visibility(sc, cam, None)
    _check_visibility(got, want, with_dom=False)


def test_clear_sentinels(renderer):
    renderer.ensure_targets(37, 19, 7, 5)
    renderer.clear()
    renderer.clear_dom()
    assert (renderer.read(abi.BUF_CENTER) == EMPTY).all()
    assert (renderer.read(abi.BUF_CONSERVATIVE) == EMPTY).all()
    assert (renderer.read(abi.BUF_BETA) == 0xFFFFFFFF).all()
    dom = renderer.read(abi.BUF_DOM)
    assert (dom[:35] == 0xFFFFFFFF).all() and (dom[35:] == 0).all() and dom.size == 35 * 17


def test_forward_z_scene_depth_and_ao_off(renderer):
    """Forward-Z projection, a scene depth buffer that hides part of the groom,
    ambient occlusion off (raster.wgsl:93-107)."""
    sc = configs.config1(scale=0.05)
    sc.groom.ambient_occlusion = False
    v = sc.view
    sc.view = host.View(v.world_from_view, host.perspective_rh(math.pi / 4, v.width / v.height, 0.1, 5000.0),
                        v.width, v.height)
    cam, dom = sc.params()
    assert cam["pass_mode"][2] == 0
    w, h = v.width, v.height
    rng = np.random.default_rng(5)
    scene_depth = np.where(rng.random(w * h) < 0.5, np.float32(1.0), np.float32(0.9990)).astype(np.float32)
    got = _visibility(renderer, sc, cam, None, scene_depth)
    want = _oracle_visibility(sc, cam, None, scene_depth)
    _check_visibility(got, want, with_dom=False)
    assert (want["center"] != EMPTY).sum() > 50
    assert ((want["center"][want["center"] != EMPTY] & np.uint64(0x3F)) == 63).all()


def test_camera_inside_the_groom_clips_at_the_near_plane(renderer):
    """Segments behind the camera or straddling it (project_world's in_front,
    the near-plane rejection in write_pixel)."""
    sc = configs.config2(scale=0.01)
    c = (sc.mesh.bounds_min + sc.mesh.bounds_max) * 0.5
    wfv = host.looking_at(c + np.array([0, 0, 20.0], np.float32), c + np.array([0, 0, -100.0], np.float32))
    sc.view = host.View(wfv, sc.view.clip_from_view, sc.view.width, sc.view.height)
    cam, dom = sc.params()
    got = _visibility(renderer, sc, cam, dom)
    want = _oracle_visibility(sc, cam, dom)
    _check_visibility(got, want)


def test_groom_outside_the_view_is_culled(renderer):
    sc = configs.config1(scale=0.02)
    wfv = host.looking_to(np.array([0, 0, 1000.0], np.float32), np.array([0, 0, 1.0], np.float32), (0, 1, 0))
    sc.view = host.View(wfv, sc.view.clip_from_view, sc.view.width, sc.view.height)
    cam, dom = sc.params()
    got = _visibility(renderer, sc, cam, None)
    want = _oracle_visibility(sc, cam, None)
    _check_visibility(got, want, with_dom=False)
    assert int(got["indirect"][0]) == 0 and (got["center"] == EMPTY).all()


def test_lod_levels_and_strand_thinning(renderer):
    """A far camera: bundles take several control-point levels and n_lod < strand_count."""
    sc = configs.config3(scale=0.01)
    sc.view = configs._camera(sc.view.width, sc.view.height, 6000.0)
    sc.groom.lam = 0.6
    cam, dom = sc.params()
    got = _visibility(renderer, sc, cam, dom)
    want = _oracle_visibility(sc, cam, dom)
    _check_visibility(got, want)
    lod = want["lod"]
    assert len(set(lod["control_points"][lod["n_lod"] > 0].tolist())) >= 2
    assert (lod["n_lod"] < lod["strand_count"]).any()


def test_empty_groom(renderer):
    from bevy_hair_gb300.groom import HairMesh

    sc = configs.config1(scale=0.02)
    sc.mesh = HairMesh(np.zeros(0, abi.GPU_BUNDLE), np.zeros(0, abi.GPU_LAYER), np.zeros((0, 4), np.float32),
                       np.zeros(3, np.float32), np.zeros(3, np.float32))
    cam, dom = sc.params()
    got = _visibility(renderer, sc, cam, dom)
    assert int(got["indirect"][0]) == 0 and int(got["dom_indirect"][0]) == 0
    assert (got["center"] == EMPTY).all() and (got["cons"] == EMPTY).all()
    n = sc.dom_size[0] * sc.dom_size[1]
    assert (got["dom"][:n] == 0xFFFFFFFF).all() and (got["dom"][n:] == 0).all()


@pytest.mark.parametrize("name", list(_scenes()))
def test_shade_filter_composite_within_tolerance(renderer, name):
    """Shade, filter and composite on identical inputs: the GPU's G-buffer and
    map go to the oracle's passes and both outputs are compared."""
    sc = _scenes()[name]()
    cam, dom = sc.params()
    lights = sc.light_array()
    w, h = sc.view.width, sc.view.height
    renderer.ensure_targets(w, h, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, lights)
    assert renderer.synchronize() == 0
    center, cons, beta = renderer.read(abi.BUF_CENTER), renderer.read(abi.BUF_CONSERVATIVE), renderer.read(abi.BUF_BETA)
    dmap = renderer.read(abi.BUF_DOM)
    shaded, sdepth = renderer.read(abi.BUF_SHADED), renderer.read(abi.BUF_SHADED_DEPTH)
    filt, fdepth = renderer.read(abi.BUF_FILTERED), renderer.read(abi.BUF_FILTERED_DEPTH)
    color, depth = renderer.read(abi.BUF_COLOR), renderer.read(abi.BUF_DEPTH)
    g.close()

    o_shaded, o_sdepth = oracle.shade(cam, center, beta, dmap, lights)
    hit = center != EMPTY
    assert hit.sum() > 50
    np.testing.assert_array_equal(sdepth, o_sdepth)
    np.testing.assert_allclose(shaded, o_shaded, rtol=SHADE_RTOL, atol=SHADE_ATOL)
    assert np.isfinite(shaded).all()

    o_filt, o_fdepth = oracle.filter_(cam, center, cons, shaded, sdepth)
    np.testing.assert_array_equal(fdepth, o_fdepth)
    np.testing.assert_array_equal(filt.reshape(-1, 4)[:, 3], o_filt.reshape(-1, 4)[:, 3])
    np.testing.assert_allclose(filt, o_filt, rtol=FILTER_RTOL, atol=FILTER_ATOL)

    o_color = np.zeros(w * h * 4, np.float32)
    o_depth = np.full(w * h, 0.0 if cam["pass_mode"][2] == 1 else 1.0, np.float32)
    oracle.composite(cam, filt, fdepth, o_color, o_depth)
    np.testing.assert_array_equal(depth, o_depth)
    np.testing.assert_allclose(color, o_color, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("scale", [0.02, 1.0])
def test_full_frame_against_the_oracle_frame(renderer, scale):
    """hg_groom_frame against the oracle's whole hair_pass sequence; at scale 1
    the benchmark frame itself, light probe included."""
    sc = configs.config2(scale=scale)
    cam, dom = sc.params()
    lights = sc.light_array()
    env = None
    if scale == 1.0:
        from bevy_hair_gb300 import envmap

        env = envmap.procedural()
    renderer.set_environment(env)
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, lights)
    assert renderer.synchronize() == 0
    renderer.set_environment(None)
    want = oracle.frame(sc.mesh, cam, dom, lights, env=env)
    _assert_equal("center", renderer.read(abi.BUF_CENTER), want["center"])
    _assert_equal("conservative", renderer.read(abi.BUF_CONSERVATIVE), want["cons"])
    _assert_equal("beta", renderer.read(abi.BUF_BETA), want["beta"])
    _assert_equal("dom", renderer.read(abi.BUF_DOM), want["dom"])
    np.testing.assert_allclose(renderer.read(abi.BUF_SHADED), want["shaded"], rtol=SHADE_RTOL, atol=SHADE_ATOL)
    color = renderer.read(abi.BUF_COLOR)
    # colour differences from shading propagate through the filter and blend
    np.testing.assert_allclose(color, want["color"], rtol=5 * SHADE_RTOL, atol=10 * SHADE_ATOL)
    g.close()


def test_light_kinds(renderer):
    """Point, spot, directional (DOM) and rect lights, given out of kind order."""
    sc = configs.config1(scale=0.05)
    cam, dom = sc.params()
    c = (sc.mesh.bounds_min + sc.mesh.bounds_max) * 0.5
    lights = pack_lights([
        Light(kind=abi.LIGHT_RECT, color=(2.0, 2.0, 2.0), position=tuple((c + [0, 400, 300]).tolist()),
              right=(1, 0, 0), up=(0, 0.6, -0.8), width=200.0, height=100.0, range=2000.0),
        Light(kind=abi.LIGHT_SPOT, color=(8e4, 6e4, 4e4), position=tuple((c + [300, 100, 300]).tolist()),
              direction=tuple((-np.array([300, 100, 300]) / np.linalg.norm([300, 100, 300])).tolist()),
              spot_scale=4.0, spot_offset=-2.5, range=1500.0),
        Light(kind=abi.LIGHT_DIRECTIONAL, color=(1.0, 1.0, 1.0), direction=(0.0, 1.0, 0.0), casts_shadows=False),
        Light(kind=abi.LIGHT_POINT, color=(5e4, 5e4, 5e4), position=tuple((c + [-300, 0, 200]).tolist()),
              range=1000.0),
        Light(kind=abi.LIGHT_DIRECTIONAL, color=(3.0, 3.0, 3.0), direction=configs.KEY_DIR, casts_shadows=True),
    ])
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, lights, exposure=0.7)
    assert renderer.synchronize() == 0
    center, beta, dmap = renderer.read(abi.BUF_CENTER), renderer.read(abi.BUF_BETA), renderer.read(abi.BUF_DOM)
    o_shaded, _ = oracle.shade(cam, center, beta, dmap, lights, exposure=0.7)
    np.testing.assert_allclose(renderer.read(abi.BUF_SHADED), o_shaded, rtol=SHADE_RTOL, atol=SHADE_ATOL)
    g.close()


def test_invalid_arguments_are_rejected(renderer):
    import ctypes as C

    lib = renderer.lib
    sc = configs.config1(scale=0.02)
    bad = sc.mesh.bundles.copy()
    bad[0]["layer_offset"] = len(sc.mesh.layers)  # past the end
    out = C.c_void_p()
    st = lib.hg_groom_upload(renderer.ctx, bad.ctypes.data, len(bad), sc.mesh.layers.ctypes.data,
                             len(sc.mesh.layers), sc.mesh.style.ctypes.data, len(sc.mesh.style), C.byref(out))
    assert st == abi.HG_INVALID_ARG and not out.value
    bad = sc.mesh.bundles.copy()
    bad[-1]["style_offset"] = len(sc.mesh.style) - 1
    st = lib.hg_groom_upload(renderer.ctx, bad.ctypes.data, len(bad), sc.mesh.layers.ctypes.data,
                             len(sc.mesh.layers), sc.mesh.style.ctypes.data, len(sc.mesh.style), C.byref(out))
    assert st == abi.HG_INVALID_ARG
    cam, dom = sc.params()
    renderer.ensure_targets(sc.view.width + 1, sc.view.height, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    with pytest.raises(abi.HairGbError) as e:
        renderer.raster(g, cam, abi.SLOT_CAMERA)  # params screen differs from the targets
    assert e.value.status == abi.HG_INVALID_ARG
    renderer.ensure_targets(sc.view.width, sc.view.height, sc.dom_size[0] + 1, sc.dom_size[1])
    with pytest.raises(abi.HairGbError):
        renderer.raster(g, dom, abi.SLOT_DOM)  # DOM params vs map size
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    many = pack_lights([Light(kind=abi.LIGHT_POINT, color=(1, 1, 1))] * (abi.MAX_LIGHTS + 1))
    with pytest.raises(abi.HairGbError) as e:
        renderer.shade(cam, many)
    assert e.value.status == abi.HG_CAPACITY_EXCEEDED
    odd = pack_lights([Light(kind=7, color=(1, 1, 1))])
    with pytest.raises(abi.HairGbError):
        renderer.shade(cam, odd)
    with pytest.raises(abi.HairGbError):
        renderer.ensure_targets(0, 10, 0, 0)
    assert renderer.synchronize() == 0
    g.close()


def test_hair_visibility_for_receivers(renderer):
    """The deep-opacity lookup other surfaces use (hair_shadow.wesl:30-75) on
    the frame's map, against the oracle, for points through the groom."""
    import ctypes as C

    import torch

    sc = configs.config1(scale=0.05)
    cam, dom = sc.params()
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, sc.light_array())
    light = np.zeros((), dtype=abi.SHADOW_LIGHT)
    assert renderer.lib.hg_shadow_light_from(dom.ctypes.data, light.ctypes.data) == abi.HG_OK
    rng = np.random.default_rng(3)
    lo, hi = sc.mesh.bounds_min - 20, sc.mesh.bounds_max + 20
    pts = np.concatenate([rng.uniform(lo, hi, size=(4000, 3)), np.ones((4000, 1))], axis=1).astype(np.float32)
    d_pts = torch.from_numpy(pts).cuda()
    d_out = torch.empty(len(pts), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = renderer.lib.hg_hair_visibility(renderer.ctx, light.ctypes.data, C.c_void_p(d_pts.data_ptr()), len(pts),
                                         C.c_void_p(d_out.data_ptr()))
    assert st == abi.HG_OK
    renderer.synchronize()
    got = d_out.cpu().numpy()
    dmap = renderer.read(abi.BUF_DOM)
    want = oracle.hair_visibility(np.atleast_1d(light).view(np.float32), dmap, *sc.dom_size, pts)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
    assert (want < 0.99).sum() > 100 and (want == 1.0).sum() > 100  # shadowed and unshadowed points
    g.close()


def test_async_readback_lands_before_the_next_frame_writes(renderer):
    """hg_copy_out_async: a frame's colour and depth copied on the copy stream
    while the next frame (another camera) is already enqueued; the next
    frame's writes wait for the copies on the device."""
    torch = pytest.importorskip("torch")
    sc = configs.config2(scale=0.02)
    cam_a, dom_a = sc.params()
    lights = sc.light_array()
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam_a, dom_a, lights)
    want_color, want_depth = renderer.read(abi.BUF_COLOR).copy(), renderer.read(abi.BUF_DEPTH).copy()
    sc.view = configs._camera(sc.view.width, sc.view.height, 700.0, azimuth=1.1)
    cam_b, dom_b = sc.params()
    color = torch.empty(want_color.size, dtype=torch.float32, pin_memory=True)
    depth = torch.empty(want_depth.size, dtype=torch.float32, pin_memory=True)
    renderer.render_groom(g, cam_a, dom_a, lights)
    renderer.read_async(abi.BUF_COLOR, color.data_ptr(), color.numel() * 4)
    renderer.read_async(abi.BUF_DEPTH, depth.data_ptr(), depth.numel() * 4)
    renderer.render_groom(g, cam_b, dom_b, lights)
    renderer.copy_wait()
    assert renderer.synchronize() == 0
    np.testing.assert_array_equal(color.numpy(), want_color)
    np.testing.assert_array_equal(depth.numpy(), want_depth)
    other = renderer.read(abi.BUF_COLOR)
    assert np.abs(other - want_color).max() > 1e-3  # frame B did overwrite the target
    with pytest.raises(abi.HairGbError):
        renderer.read_async(abi.BUF_COLOR, color.data_ptr(), 16)
    g.close()


@pytest.mark.parametrize("model", [abi.SHADE_KARIS, abi.SHADE_SURROGATE_COMPACT])
def test_orthographic_camera(renderer, model):
    """An orthographic camera: visibility bit-exact, and the shade pass's view
    direction the camera axis (hg_shade_desc.ortho), against the oracle."""
    from bevy_hair_gb300 import surrogate as S

    sc = configs.config1(scale=0.05)
    w, h = sc.view.width, sc.view.height
    ext = float(np.max(np.asarray(sc.mesh.bounds_max) - np.asarray(sc.mesh.bounds_min)))
    half = 0.6 * ext
    proj = host.orthographic_rh(-half * w / h, half * w / h, -half, half, 1.0, 4000.0)
    view = host.View(sc.view.world_from_view, proj, w, h)
    cam, dom = host.groom_params(view, sc.groom, sc.mesh.bounds_min, sc.mesh.bounds_max, sc.mesh.bundle_count,
                                 sc.directionals, sc.dom_size)
    got = _visibility(renderer, sc, cam, dom)
    want = _oracle_visibility(sc, cam, dom)
    assert (want["center"] != EMPTY).sum() > 100
    _check_visibility(got, want)
    lights = sc.light_array()
    s, mlp, arch = None, None, abi.MLP_ARCH_DEEP
    if model == abi.SHADE_SURROGATE_COMPACT:
        arch = abi.MLP_ARCH_COMPACT
        mlp = S.load_params(arch)
        s = S.Surrogate(renderer, mlp, arch)
        renderer.bind_surrogate(s)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, lights, ortho=True, model=model)
    assert renderer.synchronize() == 0
    center = renderer.read(abi.BUF_CENTER)
    _assert_equal("center", center, want["center"])
    shaded = renderer.read(abi.BUF_SHADED)
    o_shaded, _ = oracle.shade(cam, center, renderer.read(abi.BUF_BETA), renderer.read(abi.BUF_DOM), lights,
                               ortho=True, mlp=mlp, mlp_arch=arch)
    hit = center != EMPTY
    got4, want4 = shaded.reshape(-1, 4)[hit, :3], o_shaded.reshape(-1, 4)[hit, :3]
    if model == abi.SHADE_KARIS:
        np.testing.assert_allclose(shaded, o_shaded, rtol=SHADE_RTOL, atol=SHADE_ATOL)
    else:
        assert np.abs(got4 - want4).sum() / np.abs(want4).sum() < 2e-3
    # the perspective view direction gives a different picture
    o_persp, _ = oracle.shade(cam, center, renderer.read(abi.BUF_BETA), renderer.read(abi.BUF_DOM), lights,
                              ortho=False, mlp=mlp, mlp_arch=arch)
    assert np.abs(o_persp.reshape(-1, 4)[hit, :3] - want4).max() > 1e-3
    if s is not None:
        renderer.bind_surrogate(None)
        s.close()
    g.close()


@pytest.mark.parametrize("name", ["config1", "config2", "config3"])
def test_full_size_visibility_bit_exact(renderer, name):
    """The configurations at full size (config 2 is the benchmark workload:
    100k strands, 1920x1080, DOM 1024^2): LOD records, refs, G-buffer words
    and both DOM passes equal to the oracle's."""
    sc = getattr(configs, name)(scale=1.0)
    cam, dom = sc.params()
    got = _visibility(renderer, sc, cam, dom)
    want = _oracle_visibility(sc, cam, dom)
    assert (want["center"] != EMPTY).sum() > 20_000
    _check_visibility(got, want)


def test_dom_pass_over_part_of_the_bundles(renderer):
    """A DOM view over the first half of the bundles (pass_mode.y): the depth
    pass cannot use the hashed order of a full draw and must fall back to the
    refs' own order; the map stays bit-exact."""
    sc = configs.config2(scale=0.02)
    cam, dom = sc.params()
    dom = dom.copy()
    dom["pass_mode"][1] = max(1, sc.mesh.bundle_count // 2)
    got = _visibility(renderer, sc, cam, dom)
    want = _oracle_visibility(sc, cam, dom)
    assert int(got["dom_indirect"][0]) < sc.mesh.strand_count()
    assert (want["dom_depth"][: sc.dom_size[0] * sc.dom_size[1]] != 0xFFFFFFFF).any()
    _check_visibility(got, want)


def _camera_scenes():
    """Scenes for the two camera raster kinds: a plain one, deep overdraw, the
    camera inside the groom (segments cut by the near plane span the screen
    and take the long-segment path), a close-up whose segments cross several
    32x32 tiles, and forward Z with a scene depth buffer."""
    def inside():
        sc = configs.config2(scale=0.01)
        c = (sc.mesh.bounds_min + sc.mesh.bounds_max) * 0.5
        wfv = host.looking_at(c + np.array([0, 0, 20.0], np.float32), c + np.array([0, 0, -100.0], np.float32))
        sc.view = host.View(wfv, sc.view.clip_from_view, sc.view.width, sc.view.height)
        return sc, None

    def close_up():
        sc = configs.config1(scale=0.05)
        sc.view = configs._camera(1024, 768, 160.0)
        return sc, None

    def dense():
        sc = configs.config2(scale=0.25)
        sc.view = configs._camera(384, 216, 900.0)
        sc.dom_size = (192, 192)
        return sc, None

    def scene_depth():
        sc = configs.config1(scale=0.05)
        v = sc.view
        sc.view = host.View(v.world_from_view, host.perspective_rh(math.pi / 4, v.width / v.height, 0.1, 5000.0),
                            v.width, v.height)
        rng = np.random.default_rng(6)
        depth = np.where(rng.random(v.width * v.height) < 0.5, np.float32(1.0), np.float32(0.9990))
        return sc, depth.astype(np.float32)

    return {"config3": lambda: (configs.config3(scale=0.01), None), "inside": inside, "close_up": close_up,
            "dense": dense, "scene_depth": scene_depth}


@pytest.mark.parametrize("mode", [abi.CAMERA_RASTER_BINNED, abi.CAMERA_RASTER_DIRECT])
@pytest.mark.parametrize("name", list(_camera_scenes()))
def test_camera_raster_kinds_bit_exact(renderer, name, mode):
    """hg_set_camera_raster: the binned pass (tiles resolved in shared memory)
    and the direct pass (global atomics) both give the oracle's G-buffer."""
    sc, scene_depth = _camera_scenes()[name]()
    cam, _ = sc.params()
    renderer.set_camera_raster(mode)
    try:
        got = _visibility(renderer, sc, cam, None, scene_depth)
    finally:
        renderer.set_camera_raster(abi.CAMERA_RASTER_DIRECT)
    want = _oracle_visibility(sc, cam, None, scene_depth)
    assert (want["center"] != EMPTY).sum() > 50
    _check_visibility(got, want, with_dom=False)


def test_set_camera_raster_rejects_unknown_modes(renderer):
    assert renderer.lib.hg_set_camera_raster(renderer.ctx, 7) == abi.HG_INVALID_ARG


_REF = os.environ.get("BEVY_HAIR_REFERENCE")


@pytest.mark.skipif(not _REF or not (Path(_REF) / "assets" / "hair" / "woman.obj").exists(),
                    reason="the reference's grooms are not present (set BEVY_HAIR_REFERENCE)")
@pytest.mark.parametrize("name", ["wStraight", "wCurly"])
def test_reference_groom_frame_against_the_oracle(renderer, name):
    """A real groom (the reference's Yuksel asset, 50,000 strands, baked
    against woman.obj) through hg_groom_frame at 960x540: LOD records, G-buffer
    words and the deep opacity map bit-exact with the oracle's frame, colour
    within the shading tolerance."""
    hair = Path(_REF) / "assets" / "hair"
    if not (hair / f"{name}.hair").exists():
        pytest.skip(f"{name}.hair is not present")
    sc = configs.real_groom(hair / f"{name}.hair", hair / "woman.obj", 960, 540, 512)
    cam, dom = sc.params()
    lights = sc.light_array()
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, lights)
    assert renderer.synchronize() == 0
    want = oracle.frame(sc.mesh, cam, dom, lights)
    _assert_equal("center", renderer.read(abi.BUF_CENTER), want["center"])
    _assert_equal("conservative", renderer.read(abi.BUF_CONSERVATIVE), want["cons"])
    _assert_equal("beta", renderer.read(abi.BUF_BETA), want["beta"])
    _assert_equal("dom", renderer.read(abi.BUF_DOM), want["dom"])
    assert (want["center"] != EMPTY).sum() > 20_000
    np.testing.assert_allclose(renderer.read(abi.BUF_SHADED), want["shaded"], rtol=2e-3, atol=1e-5)
    g.close()
