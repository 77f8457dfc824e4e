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
