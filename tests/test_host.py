"""Host-side uniform math (src/render/pass.rs:676-787) and scene setup."""
import math

import numpy as np
import pytest

from bevy_hair_gb300 import configs, host


def test_reverse_z_detection():
    eye = host.looking_at((0, 0, 10), (0, 0, 0))
    view = host.inverse(eye)
    rev = host.perspective_infinite_reverse_rh(math.pi / 4, 1.0, 0.1) @ view
    fwd = host.perspective_rh(math.pi / 4, 1.0, 0.1, 100.0) @ view
    cam, f = np.array([0, 0, 10], np.float32), np.array([0, 0, -1], np.float32)
    assert host.depth_is_reverse(rev, cam, f)
    assert not host.depth_is_reverse(fwd, cam, f)


def test_key_direction_prefers_the_shadow_caster():
    a = host.Directional(np.array([1, 0, 0], np.float32), False)
    b = host.Directional(np.array([0, 0, 2], np.float32), True)
    assert np.allclose(host.key_direction([a, b]), [0, 0, 1])
    assert np.allclose(host.key_direction([a]), [1, 0, 0])
    d = host.key_direction([])
    assert np.allclose(d, np.array([0.35, 0.82, 0.45]) / np.linalg.norm([0.35, 0.82, 0.45]), atol=1e-6)


def test_light_fit_frames_the_groom():
    bmin, bmax = np.array([-1, -2, -3], np.float32), np.array([1, 2, 3], np.float32)
    eye, fwd, clip, near, far = host.light_fit(bmin, bmax, np.eye(4, dtype=np.float32), np.array([0, 1, 0]))
    assert near >= 0.05 and far >= near + 1.0
    assert np.allclose(fwd, [0, -1, 0])
    # every corner projects inside the orthographic light frustum
    for c in host.world_corners(bmin, bmax, np.eye(4, dtype=np.float32)):
        p = clip @ np.append(c, 1.0)
        assert np.all(np.abs(p[:2] / p[3]) <= 1.0 + 1e-5)
        d = float(np.dot(c - eye, fwd))
        assert near <= d <= far


def test_world_extent_radius_at_least_one():
    c, r = host.world_extent(np.zeros(3, np.float32), np.zeros(3, np.float32), np.eye(4, dtype=np.float32))
    assert r == 1.0 and np.allclose(c, 0)


def test_groom_params_layout():
    sc = configs.config1(scale=0.01)
    cam, dom = sc.params()
    assert cam["pass_mode"][0] == 0 and dom["pass_mode"][0] == 1 and dom["pass_mode"][3] == 1
    assert cam["pass_mode"][1] == sc.mesh.bundle_count
    assert cam["screen"][0] == sc.view.width and cam["screen"][2] == pytest.approx(0.05)
    assert dom["screen"][0] == sc.dom_size[0] and dom["dom_info"][0] == sc.dom_size[0]
    assert cam["filter_params"][3] == pytest.approx(0.05)
    assert cam["flags"].tolist() == [0, 1, 1, 1]  # config 1: LOD off
    assert cam["pass_mode"][2] == 1  # reverse-Z perspective
    lp = host.dom_layers_params(dom)
    assert lp["pass_mode"][0] == 2 and dom["pass_mode"][0] == 1


def test_shadow_light_published_from_the_dom_params():
    """hg_shadow_light_from: the ShadowLight of src/render/pass.rs:574-579."""
    from bevy_hair_gb300 import abi

    sc = configs.config1(scale=0.01)
    cam, dom = sc.params()
    light = np.zeros((), dtype=abi.SHADOW_LIGHT)
    assert abi.load().hg_shadow_light_from(dom.ctypes.data, light.ctypes.data) == abi.HG_OK
    assert np.array_equal(light["light_clip_from_world"], dom["light_clip_from_world"])
    assert light["light_eye"][3] == 1.0 and light["light_forward"][3] == 0.0
    assert np.array_equal(light["light_eye"][:3], dom["light_eye"][:3])
    assert light["depth"].tolist() == pytest.approx([dom["dom_info"][2], dom["dom_info"][3], 0.05, 1.0])
    assert abi.load().hg_shadow_light_from(cam.ctypes.data, light.ctypes.data) == abi.HG_INVALID_ARG


def _numpy_params(sc):
    return host.groom_params_numpy(sc.view, sc.groom, sc.mesh.bounds_min, sc.mesh.bounds_max, sc.mesh.bundle_count,
                                   sc.directionals, sc.dom_size)


@pytest.mark.parametrize("name", ["config1", "config2", "config3", "forward_z", "rotated_groom", "no_lights"])
def test_native_params_match_the_numpy_restatement(name):
    """hg_groom_params (native, the product path) against the NumPy restatement
    of the same host math: integer fields equal, float fields within 1e-6 of the
    largest magnitude of their vector or matrix."""
    if name == "config1":
        sc = configs.config1(scale=0.01)
    elif name == "config3":
        sc = configs.config3(scale=0.01)
    else:
        sc = configs.config2(scale=0.01)
    if name == "forward_z":
        v = sc.view
        sc.view = host.View(v.world_from_view, host.perspective_rh(math.pi / 3, v.width / v.height, 0.5, 3000.0),
                            v.width, v.height)
    if name == "rotated_groom":
        c, s = math.cos(0.7), math.sin(0.7)
        m = np.eye(4, dtype=np.float32)
        m[:3, :3] = [[c, 0, s], [0, 1, 0], [-s, 0, c]]
        m[:3, 3] = [12.0, -30.0, 5.0]
        sc.groom.world_from_model = m
    if name == "no_lights":
        sc.directionals = []
    got = sc.params()
    want = _numpy_params(sc)
    for g, w in zip(got, want):
        for f in w.dtype.names:
            a, b = np.asarray(g[f]), np.asarray(w[f])
            if a.dtype.kind == "u":
                assert np.array_equal(a, b), f
            else:
                tol = 1e-6 * max(float(np.abs(b).max()), 1e-30)
                assert np.abs(a.astype(np.float64) - b).max() <= tol, (f, a, b)
    if name == "forward_z":
        assert got[0]["pass_mode"][2] == 0
    if name == "no_lights":
        d = np.array([0.35, 0.82, 0.45]) / np.linalg.norm([0.35, 0.82, 0.45])
        assert np.allclose(-got[1]["camera_forward"][:3], d, atol=1e-6)


def test_native_params_reject_an_empty_target():
    sc = configs.config1(scale=0.01)
    sc.view = host.View(sc.view.world_from_view, sc.view.clip_from_view, 0, sc.view.height)
    with pytest.raises(ValueError):
        sc.params()
