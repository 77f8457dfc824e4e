"""Host-side uniform math of the hair pass, in f32.

Mirrors the parts of ``src/render/pass.rs`` that run on the CPU each frame:
``make_params`` (:676-709), ``key_direction`` (:711-719), ``world_corners`` /
``world_extent`` (:721-745), ``light_fit`` (:747-776), ``depth_is_reverse`` /
``clip_z`` (:778-787) and the per-groom camera/DOM parameter setup
(:399-453).  Matrices are 4x4 numpy arrays in row/column math order
(``m[row, col]``); ``cols()`` flattens them column-major as glam's
``to_cols_array_2d`` does for the uniform buffer.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from .abi import HAIR_PARAMS, LAYER_COUNT

F = np.float32
DOM_SIGMA = F(0.05)  # src/render/pass.rs:26


def v3(x, y=None, z=None) -> np.ndarray:
    if y is None:
        return np.asarray(x, dtype=F).reshape(3)
    return np.array([x, y, z], dtype=F)


def normalize_or(v: np.ndarray, fallback) -> np.ndarray:
    v = np.asarray(v, dtype=F)
    n = F(np.sqrt(np.dot(v, v)))
    if np.isfinite(n) and n > 0:
        return (v / n).astype(F)
    return v3(fallback)


def cols(m: np.ndarray) -> np.ndarray:
    return np.asarray(m, dtype=F).T.reshape(16).copy()


def transform_point(m: np.ndarray, p) -> np.ndarray:
    r = m.astype(F) @ np.append(np.asarray(p, dtype=F), F(1))
    return r[:3].astype(F)


def transform_vector(m: np.ndarray, v) -> np.ndarray:
    return (m[:3, :3].astype(F) @ np.asarray(v, dtype=F)).astype(F)


def translation(t) -> np.ndarray:
    m = np.eye(4, dtype=F)
    m[:3, 3] = np.asarray(t, dtype=F)
    return m


def looking_to(eye, direction, up) -> np.ndarray:
    """world_from_view of a transform at ``eye`` whose -Z looks along ``direction``."""
    back = normalize_or(-np.asarray(direction, dtype=F), (0, 0, 1))
    right = normalize_or(np.cross(np.asarray(up, dtype=F), back), (1, 0, 0))
    up2 = np.cross(back, right).astype(F)
    m = np.eye(4, dtype=F)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = right, up2, back, np.asarray(eye, dtype=F)
    return m


def looking_at(eye, target, up=(0, 1, 0)) -> np.ndarray:
    return looking_to(eye, np.asarray(target, dtype=F) - np.asarray(eye, dtype=F), up)


def perspective_infinite_reverse_rh(fov_y: float, aspect: float, near: float) -> np.ndarray:
    """Reverse-Z infinite perspective, the default projection of a 3-D camera."""
    f = F(1.0 / np.tan(0.5 * fov_y))
    m = np.zeros((4, 4), dtype=F)
    m[0, 0] = f / F(aspect)
    m[1, 1] = f
    m[2, 3] = F(near)
    m[3, 2] = F(-1)
    return m


def perspective_rh(fov_y: float, aspect: float, near: float, far: float) -> np.ndarray:
    """Forward-Z perspective with a [0, 1] depth range."""
    f = F(1.0 / np.tan(0.5 * fov_y))
    r = F(far / (near - far))
    m = np.zeros((4, 4), dtype=F)
    m[0, 0] = f / F(aspect)
    m[1, 1] = f
    m[2, 2] = r
    m[2, 3] = r * F(near)
    m[3, 2] = F(-1)
    return m


def orthographic_rh(left, right, bottom, top, near, far) -> np.ndarray:
    rw = F(1.0) / F(right - left)
    rh = F(1.0) / F(top - bottom)
    r = F(1.0) / F(near - far)
    m = np.eye(4, dtype=F)
    m[0, 0] = rw + rw
    m[1, 1] = rh + rh
    m[2, 2] = r
    m[0, 3] = -F(left + right) * rw
    m[1, 3] = -F(top + bottom) * rh
    m[2, 3] = r * F(near)
    return m


def inverse(m: np.ndarray) -> np.ndarray:
    return np.linalg.inv(m.astype(np.float64)).astype(F)


def clip_z(clip: np.ndarray, point) -> F:
    c = clip.astype(F) @ np.append(np.asarray(point, dtype=F), F(1))
    return F(c[2] / max(F(c[3]), F(1e-5)))


def depth_is_reverse(clip: np.ndarray, camera, forward) -> bool:
    """src/render/pass.rs:778-782"""
    camera = np.asarray(camera, dtype=F)
    forward = np.asarray(forward, dtype=F)
    return bool(clip_z(clip, camera + forward * F(0.5)) > clip_z(clip, camera + forward * F(30.0)))


@dataclass
class Directional:
    """A directional light as extract_hair sees it (src/render/mod.rs:104-107)."""
    direction_to_light: np.ndarray
    casts_shadows: bool = True


def key_direction(lights: list[Directional]) -> np.ndarray:
    """src/render/pass.rs:711-719"""
    pick = next((l for l in lights if l.casts_shadows), lights[0] if lights else None)
    d = v3(pick.direction_to_light) if pick is not None else v3(0.35, 0.82, 0.45)
    return normalize_or(d, (0, 1, 0))


def world_corners(bounds_min, bounds_max, world_from_model) -> list[np.ndarray]:
    """src/render/pass.rs:721-735"""
    out = []
    for x in (bounds_min[0], bounds_max[0]):
        for y in (bounds_min[1], bounds_max[1]):
            for z in (bounds_min[2], bounds_max[2]):
                out.append(transform_point(world_from_model, (x, y, z)))
    return out


def world_extent(bounds_min, bounds_max, world_from_model) -> tuple[np.ndarray, F]:
    """src/render/pass.rs:737-745"""
    corners = world_corners(bounds_min, bounds_max, world_from_model)
    center = (np.sum(corners, axis=0, dtype=F) / F(len(corners))).astype(F)
    radius = F(1.0)
    for c in corners:
        radius = max(radius, F(np.linalg.norm(c - center)))
    return center, F(radius)


def light_fit(bounds_min, bounds_max, world_from_model, direction_to_light):
    """Orthographic light view around the groom; src/render/pass.rs:747-776.

    Returns (eye, forward, light_clip_from_world, near, far)."""
    center, radius = world_extent(bounds_min, bounds_max, world_from_model)
    to_light = normalize_or(direction_to_light, (0, 1, 0))
    forward = (-to_light).astype(F)
    eye = (center + to_light * radius).astype(F)
    near, far = F(np.finfo(np.float32).max), F(-np.finfo(np.float32).max)
    for c in world_corners(bounds_min, bounds_max, world_from_model):
        d = F(np.dot(c - eye, forward))
        near, far = min(near, d), max(far, d)
    near = max(near - radius * F(0.05), F(0.05))
    far = max(far + radius * F(0.05), near + F(1.0))
    up = (0, 0, 1) if abs(F(np.dot(forward, v3(0, 1, 0)))) > F(0.95) else (0, 1, 0)
    view = inverse(looking_to(eye, forward, up))
    proj = orthographic_rh(-radius, radius, -radius, radius, near, far)
    return eye, forward, (proj @ view).astype(F), F(near), F(far)


def srgb_to_linear(c: float) -> float:
    c = float(c)
    return c / 12.92 if c <= 0.04045 else ((c + 0.055) / 1.055) ** 2.4


@dataclass
class HairGroom:
    """Per-groom settings (src/lib.rs:32-63, defaults :49-63).  albedo is linear RGB."""
    world_from_model: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=F))
    lam: float = 3.0
    albedo: tuple = (srgb_to_linear(0.16), srgb_to_linear(0.07), srgb_to_linear(0.035))
    roughness: float = 0.2
    tilt: float = 0.08
    lod: bool = True
    filter: bool = True
    ambient_occlusion: bool = True
    deep_opacity: bool = True
    center_diameter: float = 1.0


def make_params(*, clip_from_world, world_from_clip, world_from_model, light_clip_from_world, camera_pos,
                camera_forward, screen, groom: HairGroom, light_forward, dom_near, dom_far, dom_scale, pass_mode,
                light_eye, dom_size) -> np.ndarray:
    """HairParams; src/render/pass.rs:676-709 (the DOM size is a parameter here)."""
    p = np.zeros((), dtype=HAIR_PARAMS)
    p["clip_from_world"] = cols(clip_from_world)
    p["world_from_clip"] = cols(world_from_clip)
    p["world_from_model"] = cols(world_from_model)
    p["light_clip_from_world"] = cols(light_clip_from_world)
    p["camera_pos"] = np.append(v3(camera_pos), F(1))
    p["camera_forward"] = np.append(v3(camera_forward), F(0))
    p["screen"] = np.asarray(screen, dtype=F)
    p["appearance"] = (groom.roughness, groom.tilt, groom.lam, groom.center_diameter)
    p["filter_params"] = (F(1.0), F(0.2), max(F(dom_scale), F(1e-3)), DOM_SIGMA)
    p["albedo"] = (*groom.albedo, 1.0)
    p["flags"] = (int(groom.lod), int(groom.filter), int(groom.ambient_occlusion), int(groom.deep_opacity))
    p["pass_mode"] = np.asarray(pass_mode, dtype=np.uint32)
    p["light_eye"] = np.append(v3(light_eye), F(1))
    p["light_forward"] = np.append(v3(light_forward), F(0))
    p["dom_info"] = (F(dom_size[0]), F(dom_size[1]), F(dom_near), F(dom_far))
    return p


@dataclass
class View:
    """The camera of one view: world_from_view and clip_from_view, plus the target size."""
    world_from_view: np.ndarray
    clip_from_view: np.ndarray
    width: int
    height: int


def groom_params(view: View, groom: HairGroom, bounds_min, bounds_max, bundle_count: int,
                 directionals: list[Directional], dom_size: tuple[int, int]) -> tuple[np.ndarray, np.ndarray]:
    """Camera (pass_mode 0) and DOM depth (pass_mode 1) params of one groom;
    src/render/pass.rs:342-453, computed by the library's native host code
    (``hg_groom_params``).  The DOM layers params are the DOM params with
    pass_mode.x = 2."""
    from . import abi

    v = abi.ViewDesc()
    C.memmove(v.world_from_view, cols(view.world_from_view).ctypes.data, 64)
    C.memmove(v.clip_from_view, cols(view.clip_from_view).ctypes.data, 64)
    v.width, v.height = int(view.width), int(view.height)
    g = abi.GroomDesc()
    C.memmove(g.world_from_model, cols(groom.world_from_model).ctypes.data, 64)
    for i in range(3):
        g.bounds_min[i] = float(bounds_min[i])
        g.bounds_max[i] = float(bounds_max[i])
    g.bundle_count = int(bundle_count)
    g.roughness, g.tilt, g.lambda_, g.center_diameter = (float(groom.roughness), float(groom.tilt),
                                                         float(groom.lam), float(groom.center_diameter))
    for i, a in enumerate((*groom.albedo, 1.0)):
        g.albedo[i] = float(a)
    g.lod, g.filter = int(groom.lod), int(groom.filter)
    g.ambient_occlusion, g.deep_opacity = int(groom.ambient_occlusion), int(groom.deep_opacity)
    lights = np.zeros(len(directionals), dtype=abi.DIRECTIONAL)
    for i, d in enumerate(directionals):
        lights[i]["direction_to_light"] = np.asarray(d.direction_to_light, dtype=F)
        lights[i]["casts_shadows"] = int(d.casts_shadows)
    camera = np.zeros((), dtype=HAIR_PARAMS)
    dom = np.zeros((), dtype=HAIR_PARAMS)
    st = abi.load().hg_groom_params(C.byref(v), C.byref(g), lights.ctypes.data if len(lights) else None,
                                    len(lights), int(dom_size[0]), int(dom_size[1]), camera.ctypes.data,
                                    dom.ctypes.data)
    if st != 0:
        raise ValueError(f"hg_groom_params rejected the view or groom (status {st})")
    return camera, dom


def groom_params_numpy(view: View, groom: HairGroom, bounds_min, bounds_max, bundle_count: int,
                       directionals: list[Directional], dom_size: tuple[int, int]) -> tuple[np.ndarray, np.ndarray]:
    """The same parameters restated with NumPy (a cross-check of the native
    host code; slower by two orders of magnitude)."""
    wfv = view.world_from_view.astype(F)
    camera_pos = transform_point(wfv, (0, 0, 0))
    forward = normalize_or(-transform_vector(wfv, (0, 0, 1)), (0, 0, -1))
    clip_from_world = (view.clip_from_view.astype(F) @ inverse(wfv)).astype(F)
    world_from_clip = inverse(clip_from_world)
    reverse = depth_is_reverse(clip_from_world, camera_pos, forward)
    light_eye, light_dir, light_clip, light_near, light_far = light_fit(
        bounds_min, bounds_max, groom.world_from_model, key_direction(directionals))
    center, radius = world_extent(bounds_min, bounds_max, groom.world_from_model)
    dist = max(F(np.linalg.norm(camera_pos - center)), F(0.5))
    cam_near = F(0.05)
    cam_far = max(dist + radius * F(4.0), cam_near + F(1.0))
    dom_scale = (light_far - light_near) / F(LAYER_COUNT)
    bundle_count = max(int(bundle_count), 1)
    common = dict(world_from_model=groom.world_from_model, groom=groom, light_forward=light_dir,
                  dom_near=light_near, dom_far=light_far, dom_scale=dom_scale, light_eye=light_eye,
                  dom_size=dom_size)
    camera = make_params(clip_from_world=clip_from_world, world_from_clip=world_from_clip,
                         light_clip_from_world=light_clip, camera_pos=camera_pos, camera_forward=forward,
                         screen=(view.width, view.height, cam_near, cam_far),
                         pass_mode=(0, bundle_count, int(reverse), 0), **common)
    dom = make_params(clip_from_world=light_clip, world_from_clip=inverse(light_clip),
                      light_clip_from_world=light_clip, camera_pos=light_eye, camera_forward=light_dir,
                      screen=(dom_size[0], dom_size[1], light_near, light_far),
                      pass_mode=(1, bundle_count, int(reverse), 1), **common)
    return camera, dom


def dom_layers_params(dom: np.ndarray) -> np.ndarray:
    p = dom.copy()
    p["pass_mode"][0] = 2
    return p
